// raster.cu — sm_103a kernels of the swegl render path for one view:
//
//   k_vertex       world -> view -> projection, |z'| divide     (vertex_shaders.hpp:35-52)
//   k_flags        visibility flags of triangles                 (renderer.cpp:86-185)
//   k_compact      drawable triangles -> simple list / near-clip list
//   k_walk<0>      depth walk of simple triangles: fragment keys folded with atomicMin
//   k_walk_clip<0> the same for triangles crossing the near plane (rare)
//   k_spans<0>     long spans, one warp each
//   k_walk<1>, k_walk_clip<1>, k_spans<1>   winner walk: per-pixel progress of the winner
//   k_shade        per pixel: background or the winner's colour; depth
//   k_shade_clip   winners that belong to near-clipped triangles (rare)
//
// Depth test.  The reference draws triangles in order and keeps a fragment
// when z < zbuffer (strict, src/render/renderer.cpp:489-499), so the earliest
// drawn of equal-depth fragments wins.  Each fragment here folds the 64-bit
// key (float bits of z << 32 | draw slot) into its pixel with atomicMin: z is
// above 0.001, so its bits order like the floats, and the draw slot
// (2 * draw-order triangle + clip sub-triangle) breaks ties in draw order.
// The winner walk then records, for the fragment that owns the key, the
// per-pixel and per-edge progress the reference computed for it, and the
// shade kernel rebuilds that fragment's shader state from them.
#include <cstdint>

#include "sgl_device.cuh"
#include "sgl_internal.h"
#include "sgl_shade.cuh"

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
    s.uv[g] = make_float2(p.w, q.w);
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

// Visibility flags (renderer.cpp:86-185): inside the frustum and (double sided
// or front facing, front_face_visible :72-75, on the draw-order triple).
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
    if (ds || cross_n_z(sub3(b, a), sub3(c, a)) > 0.0f) {
        f.yes[tri.x] = 1;
        f.yes[tri.y] = 1;
        f.yes[tri.z] = 1;
    }
}

// frustum_to_viewport (viewport.cpp:123-129) of a flagged vertex
__device__ __forceinline__ V3 load_vp(const ViewDev &v, const FrameDev &f, uint32_t g)
{
    const float4 n = f.ndc[g];
    return mk3(v.vm00 * n.x + v.vm03, v.vm11 * n.y + v.vm13, n.z);
}

// Rows of fill_triangle_2's scanline range, from the three screen y values:
// ceil(max y) - ceil(min y) (renderer.cpp:390-394).  Shared by the compaction
// (work classes) and the shade kernel (which trusts it to know which
// triangles had all their spans queued).
__device__ __forceinline__ int row_extent(float ya, float yb, float yc)
{
    const float lo = fminf(ya, fminf(yb, yc)), hi = fmaxf(ya, fmaxf(yb, yc));
    const int a = f2i(ceilf(lo)), b = f2i(ceilf(hi));
    return (b - a) < 0 ? 0x7FFFFFFF : (b - a);
}

__device__ __forceinline__ int row_class(int rows)
{
    return rows <= 2 ? 0 : rows <= 4 ? 1 : rows <= 8 ? 2 : rows <= kTallRows ? 3 : 4;
}

// Drawable triangles (all three vertices flagged, renderer.cpp:248-253) into
// dense lists: those crossing the near plane, and the others by row count so
// that a warp walks triangles of similar size.  Appends are aggregated per
// block in shared memory: one global atomic per list per block.
constexpr int kCompactBlock = 512;
__global__ void __launch_bounds__(kCompactBlock) k_compact(SceneDev s, ViewDev v, FrameDev f)
{
    constexpr int L = kClasses + 1; // class lists, then the near-clip list
    __shared__ uint32_t cnt[L], base[L];
    if (threadIdx.x < L)
        cnt[threadIdx.x] = 0;
    __syncthreads();
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    int list = -1;
    if (t < s.n_triangles) {
        const uint4 tri = s.tris[t];
        if (f.yes[tri.x] && f.yes[tri.y] && f.yes[tri.z]) {
            const float4 a = f.ndc[tri.x], b = f.ndc[tri.y], c = f.ndc[tri.z];
            // fill_triangle's cases (renderer.cpp:281-318): the smallest z' decides
            if (below_near(a.z) || below_near(b.z) || below_near(c.z))
                list = kClasses;
            else
                list = row_class(row_extent(v.vm11 * a.y + v.vm13, v.vm11 * b.y + v.vm13, v.vm11 * c.y + v.vm13));
        }
    }
    uint32_t pos = 0;
    const int lane = threadIdx.x & 31;
#pragma unroll
    for (int k = 0; k < L; k++) {
        const unsigned m = __ballot_sync(0xFFFFFFFFu, list == k);
        if (!m)
            continue;
        uint32_t wbase = 0;
        if (lane == 0)
            wbase = atomicAdd(&cnt[k], (uint32_t)__popc(m));
        wbase = __shfl_sync(0xFFFFFFFFu, wbase, 0);
        if (list == k)
            pos = wbase + __popc(m & ((1u << lane) - 1u));
    }
    __syncthreads();
    if (threadIdx.x < L && cnt[threadIdx.x])
        base[threadIdx.x] = atomicAdd(&f.counters32[threadIdx.x < kClasses ? C_CLASS0 + threadIdx.x : C_CLIPTRI],
                                      cnt[threadIdx.x]);
    __syncthreads();
    if (list == kClasses)
        f.cliptri[base[list] + pos] = t;
    else if (list >= 0)
        f.classes[(size_t)list * s.n_triangles + base[list] + pos] = t;
}

// ------------------------------------------------------------ triangle walk --

// fill_triangle's sort of the vertex pointers by z' descending
// (renderer.cpp:264-279), on values; pa/pb/pc track which input landed where.
__device__ __forceinline__ bool sort_z_desc(V3 &a, V3 &b, V3 &c, int &pa, int &pb, int &pc)
{
    bool inv = false;
    V3 t;
    int q;
    if (b.z > a.z) { t = a; a = b; b = t; q = pa; pa = pb; pb = q; inv = !inv; }
    if (c.z > b.z) { t = b; b = c; c = t; q = pb; pb = pc; pc = q; inv = !inv; }
    if (b.z > a.z) { t = a; a = b; b = t; q = pa; pa = pb; pb = q; inv = !inv; }
    return inv;
}

// fill_triangle_2's sort by screen y ascending (renderer.cpp:375-387)
__device__ __forceinline__ void sort_y_asc(V3 &a, V3 &b, V3 &c, int &pa, int &pb, int &pc)
{
    V3 t;
    int q;
    if (b.y < a.y) { t = a; a = b; b = t; q = pa; pa = pb; pb = q; }
    if (c.y < b.y) { t = b; b = c; c = t; q = pb; pb = pc; pc = q; }
    if (b.y < a.y) { t = a; a = b; b = t; q = pa; pa = pb; pb = q; }
}

// fill_half_triangle row loop (renderer.cpp:462-558): per row the span
// [x1, x2) clipped to the viewport goes to the visitor, then both edges step.
template <class Vis>
__device__ __forceinline__ void walk_half(const ViewDev &v, int y, int y_end, Side &Ls, Side &Rs, uint32_t bits,
                                          Vis &vis)
{
    for (; y < y_end && vis.active(); y++) {
        int x1 = f2i(ceilf(Ls.x));
        if (x1 < v.x)
            x1 = v.x;
        int x2 = f2i(ceilf(Rs.x));
        if (x2 > v.x + v.w)
            x2 = v.x + v.w;
        if (x1 < x2)
            vis.span(y, x1, x2, Ls, Rs, bits);
        Ls.x = Ls.x + Ls.ratio;
        Rs.x = Rs.x + Rs.ratio;
        Ls.it.step();
        Rs.it.step();
    }
}

// fill_triangle_2 (src/render/renderer.cpp:361-460) on screen positions, in
// the vertex order fill_triangle passes them: edge setup and both halves.
// Span bits: kBitLower for the lower half, kBitLLR for long_line_on_right.
template <class Vis>
__device__ __forceinline__ void walk_sub(const ViewDev &v, V3 a, V3 b, V3 c, Vis &vis)
{
    int pa = 0, pb = 1, pc = 2;
    sort_y_asc(a, b, c, pa, pb, pc);
    const V3 v0 = a, v1 = b, v2 = c;
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
    vis.drawn();
    if (y1 >= v.y) {
        sht.ratio = (v1.x - v0.x) / (v1.y - v0.y);
        sht.it.init_self(v1.y - v0.y, v0.z, v1.z);
        const int y = y0 > v.y ? y0 : v.y;
        const int y_end = y1 < v.y + v.h ? y1 : v.y + v.h;
        sht.it.displace((float)y - v0.y);
        sht.x = v0.x + sht.ratio * ((float)y - v0.y);
        const bool llr = lng.ratio > sht.ratio;
        const uint32_t bits = llr ? kBitLLR : 0u;
        if (llr)
            walk_half(v, y, y_end, sht, lng, bits, vis);
        else
            walk_half(v, y, y_end, lng, sht, bits, vis);
    }
    if (y1 < v.y + v.h) {
        sht.ratio = (v2.x - v1.x) / (v2.y - v1.y);
        sht.it.init_self(v2.y - v1.y, v1.z, v2.z);
        const int y = y1 > v.y ? y1 : v.y;
        const int y_end = y2 < v.y + v.h ? y2 : v.y + v.h;
        sht.it.displace((float)y - v1.y);
        sht.x = v1.x + sht.ratio * ((float)y - v1.y);
        const bool llr = lng.ratio < sht.ratio;
        const uint32_t bits = kBitLower | (llr ? kBitLLR : 0u);
        if (llr)
            walk_half(v, y, y_end, sht, lng, bits, vis);
        else
            walk_half(v, y, y_end, lng, sht, bits, vis);
    }
}

// The per-pixel loop of fill_half_triangle for one span: qpixel set up over
// the span (renderer.cpp:476-480) and stepped per pixel (:486).  `op(x, z,
// progress)` gets each pixel nearer than the near plane and the clear depth.
template <class Op>
__device__ __forceinline__ void span_pixels(int x1, int x2, const Side &Ls, const Side &Rs, Op &op)
{
    Interp q;
    q.init_self(Rs.x - Ls.x, Ls.it.value(), Rs.it.value());
    q.displace((float)x1 - Ls.x);
    for (; x1 < x2; x1++, q.step()) {
        const float z = q.value();
        if (below_near(z)) // (double)z <= 0.001
            continue;
        if (__float_as_uint(z) >= kMaxZBits)
            continue; // z >= the cleared depth never passes
        op(x1, z, q.alpha);
    }
}

__device__ __forceinline__ unsigned long long make_key(float z, uint32_t slot)
{
    return ((unsigned long long)__float_as_uint(z) << 32) | slot;
}

// Queue a long span: the qpixel state after its displacement to x1.
__device__ __forceinline__ bool enqueue_span(const FrameDev &f, uint32_t slot, int y, int x1, int x2, const Side &Ls,
                                             const Side &Rs, uint32_t bits)
{
    const uint32_t i = atomicAdd(&f.counters32[C_SPANS], 1u);
    if (i >= f.span_cap) {
        atomicExch(&f.counters32[C_OVERFLOW], 1u);
        return false;
    }
    Interp q;
    q.init_self(Rs.x - Ls.x, Ls.it.value(), Rs.it.value());
    q.displace((float)x1 - Ls.x);
    SpanRec r;
    r.slot = slot;
    r.y_bits = (uint32_t)y | bits;
    r.x1 = x1;
    r.x2 = x2;
    r.top = q.top;
    r.tstep = q.tstep;
    r.bottom = q.bottom;
    r.bstep = q.bstep;
    r.v0 = q.v0;
    r.dv = q.dv;
    r.progL = Ls.it.alpha;
    r.progR = Rs.it.alpha;
    f.spans[i] = r;
    return true;
}

struct DepthVisitor {
    const ViewDev &v;
    const FrameDev &f;
    uint32_t slot;
    unsigned long long drawn_n, fragments;
    bool queue_all; // tall triangle: every span goes to the span kernels

    __device__ __forceinline__ bool active() const { return true; }
    __device__ __forceinline__ void drawn()
    {
        drawn_n++;
        if (f.slot_flags)
            f.slot_flags[slot] = 1;
    }
    __device__ __forceinline__ void span(int y, int x1, int x2, const Side &Ls, const Side &Rs, uint32_t bits)
    {
        fragments += (unsigned long long)(x2 - x1);
        if ((queue_all || x2 - x1 > kInlineSpan) && enqueue_span(f, slot, y, x1, x2, Ls, Rs, bits))
            return;
        unsigned long long *row = f.key + ((long long)(y - v.y) * v.w - v.x);
        const uint32_t sl = slot;
        auto op = [&](int x, float z, float) {
            atomicMin(row + x, make_key(z, sl)); // result unused: a reduction, no round trip
        };
        span_pixels(x1, x2, Ls, Rs, op);
    }
};

struct WinnerVisitor {
    const ViewDev &v;
    const FrameDev &f;
    uint32_t slot;
    bool long_inline; // the span queue overflowed: long spans are handled here too

    __device__ __forceinline__ bool active() const { return true; }
    __device__ __forceinline__ void drawn() {}
    __device__ __forceinline__ void span(int y, int x1, int x2, const Side &Ls, const Side &Rs, uint32_t bits)
    {
        if (x2 - x1 > kInlineSpan && !long_inline)
            return; // recorded by the winner span kernel from the queue
        const long long base = (long long)(y - v.y) * v.w - v.x;
        const unsigned long long *row = f.key + base;
        float4 *rec = f.prec + base;
        const uint32_t sl = slot;
        const float pl = Ls.it.alpha, pr = Rs.it.alpha;
        auto op = [&](int x, float z, float progress) {
            if (row[x] == make_key(z, sl))
                rec[x] = make_float4(progress, pl, pr, __uint_as_float(bits));
        };
        span_pixels(x1, x2, Ls, Rs, op);
    }
};

// Replays one triangle's walk up to pixel (tx, ty) to recover the progress
// values the reference had there: the edge progress of the row and the
// qpixel progress after (tx - x1) steps (renderer.cpp:474-493).  Spans wider
// than kInlineSpan were recorded by the span kernels instead (use_prec).
struct ReplayVisitor {
    int tx, ty;
    bool found, use_prec;
    float4 rec;

    __device__ __forceinline__ bool active() const { return !found && !use_prec; }
    __device__ __forceinline__ void drawn() {}
    __device__ __forceinline__ void span(int y, int x1, int x2, const Side &Ls, const Side &Rs, uint32_t bits)
    {
        if (y != ty || tx < x1 || tx >= x2)
            return;
        if (x2 - x1 > kInlineSpan) {
            use_prec = true;
            return;
        }
        Interp q;
        q.init_self(Rs.x - Ls.x, Ls.it.value(), Rs.it.value());
        q.displace((float)x1 - Ls.x);
        for (int x = x1; x < tx; x++)
            q.step();
        rec = make_float4(q.alpha, Ls.it.alpha, Rs.it.alpha, __uint_as_float(bits));
        found = true;
    }
};

__device__ __forceinline__ void warp_add(unsigned long long *dst, unsigned long long v)
{
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_down_sync(0xFFFFFFFFu, v, o);
    if ((threadIdx.x & 31) == 0 && v)
        atomicAdd(dst, v);
}

__device__ __forceinline__ void set_queue_all(DepthVisitor &vis, bool q) { vis.queue_all = q; }
__device__ __forceinline__ void set_queue_all(WinnerVisitor &, bool) {}

// Walk of the triangles wholly in front of the near plane: fill_triangle's
// normal case (renderer.cpp:281-285), one sub-triangle, slot 2t.  The grid
// strides over the class lists concatenated, small triangles first.
template <class Vis>
__device__ __forceinline__ void walk_simple(const SceneDev &s, const ViewDev &v, const FrameDev &f, Vis &vis,
                                            bool tall_queue)
{
    uint32_t start[kClasses + 1];
    start[0] = 0;
#pragma unroll
    for (int k = 0; k < kClasses; k++)
        start[k + 1] = start[k] + f.counters32[C_CLASS0 + k];
    const uint32_t n = start[kClasses];
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        int k = 0;
#pragma unroll
        for (int c = 1; c < kClasses; c++)
            k += (i >= start[c]) ? 1 : 0;
        const uint32_t t = f.classes[(size_t)k * s.n_triangles + (i - start[k])];
        const uint4 tri = s.tris[t];
        V3 a = load_vp(v, f, tri.x), b = load_vp(v, f, tri.y), c = load_vp(v, f, tri.z);
        int pa = 0, pb = 1, pc = 2;
        sort_z_desc(a, b, c, pa, pb, pc);
        vis.slot = 2 * t;
        set_queue_all(vis, tall_queue && k == kClasses - 1);
        walk_sub(v, a, b, c, vis);
    }
}

// Depth walk (WINNER = 0), and the winner walk (WINNER = 1) that only runs
// when the span queue overflowed (the shade kernel replays winners otherwise).
template <int WINNER>
__global__ void __launch_bounds__(128, 8) k_walk(SceneDev s, ViewDev v, FrameDev f)
{
    if (!WINNER) {
        DepthVisitor vis{v, f, 0u, 0ull, 0ull, false};
        walk_simple(s, v, f, vis, true);
        warp_add(&f.counters[C_DRAWN], vis.drawn_n);
        warp_add(&f.counters[C_FRAGMENTS], vis.fragments);
    } else {
        if (!f.counters32[C_OVERFLOW])
            return;
        WinnerVisitor vis{v, f, 0u, true};
        walk_simple(s, v, f, vis, false);
    }
}

// ------------------------------------------------------------- near clip --

// A vertex with everything fill_triangle's clip branches need (mesh_vertex_t,
// swegl/data/model.hpp:20-29).
struct TV {
    V3 vp;      // v_viewport: screen x, y and z'
    V3 world;   // v_world
    V3 normal;  // object-space normal
    V3 nworld;  // normal_world
    V2 uv;
};

__device__ __forceinline__ void load_tv(const SceneDev &s, const ViewDev &v, const FrameDev &f, uint32_t g, TV &o)
{
    o.vp = load_vp(v, f, g);
    const float4 w = s.wpos[g];
    o.world = mk3(w.x, w.y, w.z);
    const float4 nv = s.nrm_v[g];
    o.normal = mk3(nv.x, nv.y, nv.z);
    const float2 uv = s.uv[g];
    o.uv = mk2(uv.x, uv.y);
    const float4 nw = s.wnrm[g];
    o.nworld = mk3(nw.x, nw.y, nw.z);
}

// world_to_viewport (vertex_shaders.hpp:54-59) of a near-clip vertex
__device__ __forceinline__ void world_to_viewport(const ViewDev &v, TV &o, const float *rs)
{
    V3 p = transform3(o.world, v.view);
    o.nworld = normalize3(normalize3(rotate_n(o.normal, rs)));
    p = transform3(p, v.proj);
    if (p.z != 0.0f) {
        p.x = p.x / fabsf(p.z);
        p.y = p.y / fabsf(p.z);
    }
    p.x = v.vm00 * p.x + v.vm03;
    p.y = v.vm11 * p.y + v.vm13;
    o.vp = p;
}

// near-clip vertex a + (b - a) * cut (renderer.cpp:290-297)
__device__ __forceinline__ void clip_vertex(const ViewDev &v, TV &o, const TV &a, const TV &b, float cut,
                                            const float *rs)
{
    o.world = add3(a.world, mul3(sub3(b.world, a.world), cut));
    o.uv = add2(a.uv, mul2(sub2(b.uv, a.uv), cut));
    if (b.normal.x == a.normal.x && b.normal.y == a.normal.y && b.normal.z == a.normal.z)
        o.normal = a.normal;
    else
        o.normal = normalize3(add3(a.normal, mul3(sub3(b.normal, a.normal), cut)));
    world_to_viewport(v, o, rs);
}

// fill_triangle (src/render/renderer.cpp:240-359) for a triangle with a vertex
// behind the near plane: calls emit(slot, a, b, c, front_face_visible) for the
// fill_triangle_2 calls it makes, in order.  Only the rare near-clip triangles
// come here, so its register and stack use stay off the common walk.
template <class Emit>
__device__ __forceinline__ void clip_triangle(const SceneDev &s, const ViewDev &v, const FrameDev &f, uint32_t t,
                                              Emit &emit)
{
    const uint4 tri = s.tris[t];
    TV tv[3];
    load_tv(s, v, f, tri.x, tv[0]);
    load_tv(s, v, f, tri.y, tv[1]);
    load_tv(s, v, f, tri.z, tv[2]);
    const float *rs = s.node_rs + 16 * s.prims[tri.w].node;
    const TV *a = &tv[0], *b = &tv[1], *c = &tv[2], *tp;
    bool ffv = cross_n_z(sub3(b->vp, a->vp), sub3(c->vp, a->vp)) < 0.0f;
    bool inverted_order = false;
    if (b->vp.z > a->vp.z) { tp = a; a = b; b = tp; inverted_order = !inverted_order; }
    if (c->vp.z > b->vp.z) { tp = b; b = c; c = tp; inverted_order = !inverted_order; }
    if (b->vp.z > a->vp.z) { tp = a; a = b; b = tp; inverted_order = !inverted_order; }
    const V3 v0 = a->vp, v1 = b->vp, v2 = c->vp;
    if (at_or_past_near(v2.z)) {
        emit(2 * t, *a, *b, *c, ffv); // not reached: compaction sent it to the simple list
    } else if (below_near(v1.z)) {
        TV n1, n2;
        clip_vertex(v, n1, *a, *b, (v0.z - 0.001f) / (v0.z - v1.z), rs);
        clip_vertex(v, n2, *a, *c, (v0.z - 0.001f) / (v0.z - v2.z), rs);
        ffv = cross_n_z(sub3(n1.vp, v0), sub3(n2.vp, v0)) < 0.0f;
        if (inverted_order)
            ffv = !ffv;
        emit(2 * t, *a, n1, n2, ffv);
    } else {
        TV n1, n2;
        clip_vertex(v, n1, *a, *c, (v0.z - 0.001f) / (v0.z - v2.z), rs);
        clip_vertex(v, n2, *b, *c, (v1.z - 0.001f) / (v1.z - v2.z), rs);
        ffv = cross_n_z(sub3(v1, v0), sub3(n2.vp, v0)) < 0.0f;
        if (inverted_order)
            ffv = !ffv;
        emit(2 * t, *a, *b, n2, ffv);
        ffv = cross_n_z(sub3(n2.vp, v0), sub3(n1.vp, v0)) < 0.0f;
        if (inverted_order)
            ffv = !ffv;
        emit(2 * t + 1, *a, n2, n1, ffv);
    }
}

template <int WINNER>
__global__ void __launch_bounds__(128) k_walk_clip(SceneDev s, ViewDev v, FrameDev f)
{
    const uint32_t n = f.counters32[C_CLIPTRI];
    const uint32_t stride = gridDim.x * blockDim.x;
    DepthVisitor dvis{v, f, 0u, 0ull, 0ull, false};
    WinnerVisitor wvis{v, f, 0u, f.counters32[C_OVERFLOW] != 0u};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        auto emit = [&](uint32_t slot, const TV &a, const TV &b, const TV &c, bool) {
            if (!WINNER) {
                dvis.slot = slot;
                walk_sub(v, a.vp, b.vp, c.vp, dvis);
            } else {
                wvis.slot = slot;
                walk_sub(v, a.vp, b.vp, c.vp, wvis);
            }
        };
        clip_triangle(s, v, f, f.cliptri[i], emit);
    }
    if (!WINNER) {
        warp_add(&f.counters[C_DRAWN], dvis.drawn_n);
        warp_add(&f.counters[C_FRAGMENTS], dvis.fragments);
    }
}

// ------------------------------------------------------------- long spans --

// Long spans, one warp each.  The qpixel chain (top += tstep, bottom +=
// bstep per pixel, interpolator.hpp:96-100) is serial in floating point, so
// every lane runs the same 32 steps and keeps the state of its own pixel; the
// divisions, depth and key work then run on all lanes.
template <int WINNER>
__global__ void __launch_bounds__(256) k_spans(ViewDev v, FrameDev f)
{
    const uint32_t n_queued = f.counters32[C_SPANS];
    const uint32_t n = n_queued < f.span_cap ? n_queued : f.span_cap;
    if (WINNER && f.counters32[C_OVERFLOW])
        return; // the winner walks handled every span inline
    const int lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t n_warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t i = warp; i < n; i += n_warps) {
        const SpanRec r = f.spans[i];
        const int y = (int)(r.y_bits & kYMask);
        const long long base = (long long)(y - v.y) * v.w - v.x;
        float top = r.top, bottom = r.bottom;
        for (int x0 = r.x1; x0 < r.x2; x0 += 32) {
            float mt = top, mb = bottom;
#pragma unroll
            for (int k = 0; k < 32; k++) {
                if (k == lane) {
                    mt = top;
                    mb = bottom;
                }
                top = top + r.tstep;
                bottom = bottom + r.bstep;
            }
            const int x = x0 + lane;
            if (x >= r.x2)
                continue;
            const float alpha = mt / mb;
            const float z = r.v0 + r.dv * alpha;
            if (below_near(z) || __float_as_uint(z) >= kMaxZBits)
                continue;
            const unsigned long long key = make_key(z, r.slot);
            unsigned long long *kp = f.key + base + x;
            if (!WINNER) {
                if (key < *kp)
                    atomicMin(kp, key);
            } else if (*kp == key) {
                f.prec[base + x] = make_float4(alpha, r.progL, r.progR, __uint_as_float(r.y_bits & ~kYMask));
            }
        }
    }
}

// ------------------------------------------------------------------ shade --

__device__ __forceinline__ void bind_material(const SceneDev &s, uint32_t prim, Shader &sh)
{
    const PrimDesc pd = s.prims[prim];
    const MatDesc m = (pd.material >= 0 && pd.material < s.n_mats) ? s.mats[pd.material] : s.default_mat;
    sh.shininess = m.shininess;
    sh.color = m.color;
    if (m.texture < 0 || m.texture >= s.n_texs) {
        sh.tex = nullptr;
        sh.tw = sh.th = 1;
    } else {
        const TexDesc td = s.texs[m.texture];
        sh.tex = td.texels;
        sh.tw = td.w;
        sh.th = td.h;
    }
}

// prepare_for_upper/lower_triangle, prepare_for_scanline and shade for the
// winner's recorded progress values (renderer.cpp:433-493)
__device__ __forceinline__ uint32_t shade_winner(Shader &sh, const LightsDev &L, const ViewDev &v, float4 rec)
{
    const uint32_t bits = __float_as_uint(rec.w);
    const bool llr = (bits & kBitLLR) != 0u;
    if (bits & kBitLower)
        sh_prepare_lower(sh, llr);
    else
        sh_prepare_upper(sh, llr);
    sh_prepare_scanline(sh, rec.y, rec.z);
    return sh_shade(sh, L, v, rec.x);
}

// Per viewport pixel: the background of viewport_t::clear (viewport.cpp:88-113)
// or the colour of the winning fragment; and the depth of every pixel.
// Winners of near-clipped triangles are passed on to k_shade_clip.
__global__ void __launch_bounds__(128) k_shade(SceneDev s, LightsDev L, ViewDev v, FrameDev f)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= v.w * v.h)
        return;
    const int y = i / v.w, x = i - y * v.w;
    const unsigned long long k = f.key[i];
    uint32_t *px = f.pixels + (long long)y * f.pitch_px + x;
    if (k == kEmptyKey) {
        *px = 0u;
        if (f.zbuf)
            f.zbuf[i] = __uint_as_float(kMaxZBits);
        return;
    }
    if (f.zbuf)
        f.zbuf[i] = __uint_as_float((uint32_t)(k >> 32));
    const uint32_t slot = (uint32_t)k;
    const uint4 tri = s.tris[slot >> 1];
    V3 a = load_vp(v, f, tri.x), b = load_vp(v, f, tri.y), c = load_vp(v, f, tri.z);
    if (below_near(a.z) || below_near(b.z) || below_near(c.z)) {
        const uint32_t j = atomicAdd(&f.counters32[C_CLIPPX], 1u);
        f.clippx[j] = (uint32_t)i; // at most one per pixel: fits the w*h list
        return;
    }
    // fill_triangle: front_face_visible, then the z sort; fill_triangle_2: the y sort
    const bool ffv = cross_n_z(sub3(b, a), sub3(c, a)) < 0.0f;
    int pa = 0, pb = 1, pc = 2;
    sort_z_desc(a, b, c, pa, pb, pc);
    float4 rec;
    if (f.counters32[C_OVERFLOW] || row_extent(a.y, b.y, c.y) > kTallRows) {
        rec = f.prec[i]; // recorded by the span kernels (or the overflow winner walk)
    } else {
        ReplayVisitor rv{x + v.x, y + v.y, false, false, make_float4(0.f, 0.f, 0.f, 0.f)};
        walk_sub(v, a, b, c, rv);
        rec = rv.found ? rv.rec : f.prec[i];
    }
    sort_y_asc(a, b, c, pa, pb, pc);
    const uint32_t g0 = pa == 0 ? tri.x : (pa == 1 ? tri.y : tri.z);
    const uint32_t g1 = pb == 0 ? tri.x : (pb == 1 ? tri.y : tri.z);
    const uint32_t g2 = pc == 0 ? tri.x : (pc == 1 ? tri.y : tri.z);
    Shader sh;
    bind_material(s, tri.w, sh);
    const float4 w0 = s.wpos[g0], w1 = s.wpos[g1], w2 = s.wpos[g2];
    const float4 n0 = s.wnrm[g0], n1 = s.wnrm[g1], n2 = s.wnrm[g2];
    const float2 u0 = s.uv[g0], u1 = s.uv[g1], u2 = s.uv[g2];
    const V3 sw[3] = {mk3(w0.x, w0.y, w0.z), mk3(w1.x, w1.y, w1.z), mk3(w2.x, w2.y, w2.z)};
    const V3 sn[3] = {mk3(n0.x, n0.y, n0.z), mk3(n1.x, n1.y, n1.z), mk3(n2.x, n2.y, n2.z)};
    const V2 su[3] = {mk2(u0.x, u0.y), mk2(u1.x, u1.y), mk2(u2.x, u2.y)};
    sh_prepare_triangle(sh, sw, sn, su, !ffv);
    *px = shade_winner(sh, L, v, rec);
}

// Winners that belong to near-clipped triangles: the clip vertices are
// rebuilt exactly as fill_triangle makes them.
__global__ void __launch_bounds__(128) k_shade_clip(SceneDev s, LightsDev L, ViewDev v, FrameDev f)
{
    const uint32_t n = f.counters32[C_CLIPPX];
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const uint32_t i = f.clippx[j];
        const int y = (int)i / v.w, x = (int)i - y * v.w;
        const uint32_t slot = (uint32_t)f.key[i];
        const float4 rec = f.prec[i];
        Shader sh;
        bool done = false;
        auto emit = [&](uint32_t sl, const TV &a, const TV &b, const TV &c, bool ffv) {
            if (sl != slot || done)
                return;
            const TV *p0 = &a, *p1 = &b, *p2 = &c, *t;
            if (p1->vp.y < p0->vp.y) { t = p0; p0 = p1; p1 = t; }
            if (p2->vp.y < p1->vp.y) { t = p1; p1 = p2; p2 = t; }
            if (p1->vp.y < p0->vp.y) { t = p0; p0 = p1; p1 = t; }
            const V3 sw[3] = {p0->world, p1->world, p2->world};
            const V3 sn[3] = {p0->nworld, p1->nworld, p2->nworld};
            const V2 su[3] = {p0->uv, p1->uv, p2->uv};
            bind_material(s, s.tris[slot >> 1].w, sh);
            sh_prepare_triangle(sh, sw, sn, su, !ffv);
            done = true;
        };
        clip_triangle(s, v, f, slot >> 1, emit);
        if (done)
            f.pixels[(long long)y * f.pitch_px + x] = shade_winner(sh, L, v, rec);
    }
}

// ---------------------------------------------------------------- launches --

static inline unsigned grid_for(uint64_t n, int block) { return (unsigned)((n + block - 1) / block); }

static int sm_count()
{
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0)
            n = 132;
    }
    return n;
}

cudaError_t launch_world(const SceneDev &s, cudaStream_t st)
{
    if (s.n_vertices == 0)
        return cudaSuccess;
    k_world<<<grid_for(s.n_vertices, 256), 256, 0, st>>>(s);
    return cudaGetLastError();
}

const char *prof_kernel_name(int k)
{
    static const char *names[kProfKernels] = {"clear",         "k_vertex",       "k_flags",
                                              "k_compact",     "k_walk_depth",   "k_spans_depth",
                                              "k_walk_winner", "k_spans_winner", "k_shade"};
    return (k >= 0 && k < kProfKernels) ? names[k] : "?";
}

// Fold the previous frame's event timings into the totals.
static void prof_collect(Profiler *p)
{
    if (!p || !p->pending)
        return;
    if (cudaEventSynchronize(p->ev[kProfKernels]) == cudaSuccess) {
        for (int k = 0; k < kProfKernels; k++) {
            float ms = 0.0f;
            if (cudaEventElapsedTime(&ms, p->ev[k], p->ev[k + 1]) == cudaSuccess) {
                p->ms[k] += ms;
                p->launches[k]++;
            }
        }
    }
    cudaGetLastError();
    p->pending = false;
}

void prof_flush(Profiler *p) { prof_collect(p); }

cudaError_t launch_frame(const SceneDev &s, const LightsDev &l, const ViewDev &v, const FrameDev &f, cudaStream_t st,
                         int *launches, Profiler *prof)
{
    int n = 0;
    const bool timed = prof && prof->enabled;
    if (timed) {
        prof_collect(prof);
        for (int k = 0; k <= kProfKernels; k++)
            if (!prof->ev[k] && cudaEventCreate(&prof->ev[k]) != cudaSuccess)
                return cudaGetLastError();
    }
    auto mark = [&](int k) {
        if (timed)
            cudaEventRecord(prof->ev[k], st);
    };
    const int sms = sm_count();
    mark(PK_CLEAR);
    cudaError_t e = cudaMemsetAsync(f.key, 0xFF, sizeof(unsigned long long) * (size_t)v.w * v.h, st);
    if (e == cudaSuccess)
        e = cudaMemsetAsync(f.counters, 0, sizeof(unsigned long long) * kCounterWords, st);
    if (e != cudaSuccess)
        return e;
    mark(PK_VERTEX);
    if (s.n_vertices) {
        k_vertex<<<grid_for(s.n_vertices, 256), 256, 0, st>>>(s, v, f);
        n++;
    }
    mark(PK_FLAGS);
    if (s.n_triangles) {
        k_flags<<<grid_for(s.n_triangles, 256), 256, 0, st>>>(s, f);
        n++;
    }
    mark(PK_COMPACT);
    if (s.n_triangles) {
        k_compact<<<grid_for(s.n_triangles, kCompactBlock), kCompactBlock, 0, st>>>(s, v, f);
        n++;
    }
    mark(PK_WALK_DEPTH);
    if (s.n_triangles) {
        k_walk<0><<<sms * 8, 128, 0, st>>>(s, v, f);
        k_walk_clip<0><<<sms, 128, 0, st>>>(s, v, f);
        n += 2;
    }
    mark(PK_SPANS_DEPTH);
    if (s.n_triangles) {
        k_spans<0><<<sms * 4, 256, 0, st>>>(v, f);
        n++;
    }
    mark(PK_WALK_WINNER);
    if (s.n_triangles) {
        k_walk<1><<<sms * 8, 128, 0, st>>>(s, v, f);
        k_walk_clip<1><<<sms, 128, 0, st>>>(s, v, f);
        n += 2;
    }
    mark(PK_SPANS_WINNER);
    if (s.n_triangles) {
        k_spans<1><<<sms * 4, 256, 0, st>>>(v, f);
        n++;
    }
    mark(PK_SHADE);
    k_shade<<<grid_for((uint64_t)v.w * v.h, 128), 128, 0, st>>>(s, l, v, f);
    n++;
    if (s.n_triangles) {
        k_shade_clip<<<sms, 128, 0, st>>>(s, l, v, f);
        n++;
    }
    if (timed) {
        cudaEventRecord(prof->ev[kProfKernels], st);
        prof->pending = true;
    }
    if (launches)
        *launches += n;
    return cudaGetLastError();
}

} // namespace sgl
