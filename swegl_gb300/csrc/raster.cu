// raster.cu — sm_103a kernels of the swegl render path.
//
// Every kernel works on a batch of views (items: scene, camera, buffers) and
// is a persistent grid-stride kernel with a fixed grid that reads the batch
// totals from device memory, so one launch sequence (and one CUDA graph)
// serves any batch.  The plain one-frame-per-launch renderer is a batch of one.
//
//   k_clear       per pixel: depth key cleared (viewport_t::clear, viewport.cpp:88-113)
//   k_vertex      world -> view -> projection, |z'| divide      (vertex_shaders.hpp:35-52)
//   k_flags       visibility flags of triangles                  (renderer.cpp:86-185)
//   k_compact     drawable triangles -> one list grouped by row class / near-clip list
//   k_walk        depth walk: fragment keys folded with atomicMin
//   k_walk_clip   the same for triangles crossing the near plane (rare)
//   k_spans<0>    long spans binned by the walk, one warp each
//   k_spans<1>, k_walk_clip<1>   winner records for binned spans and clipped triangles
//   k_walk_winner winner records of every span, only after a bin overflow
//   k_shade       per pixel: background or the winner's colour, and depth
//   k_shade_clip  winners that belong to near-clipped triangles (rare)
//   k_dof         depth-of-field gather of the items that ask for it
//
// Depth test.  The reference draws triangles in order and keeps a fragment
// when z < zbuffer (strict, src/render/renderer.cpp:489-499), so the earliest
// drawn of equal-depth fragments wins.  Each fragment here folds the 64-bit
// key (float bits of z << 32 | draw slot) into its pixel with atomicMin: z is
// above 0.001, so its bits order like the floats, and the draw slot
// (2 * draw-order triangle + clip sub-triangle) breaks ties in draw order.
// The shade kernel then replays the winner's row and pixel steps to recover
// the progress values the reference shaded with; spans too long to replay
// cheaply have them recorded by the span kernels instead.
#include <cstdint>

#include "sgl_device.cuh"
#include "sgl_dof_taps.h"
#include "sgl_internal.h"
#include "sgl_shade.cuh"

namespace sgl {

// Index of the item owning global index x: largest i with base[i] <= x.
__device__ __forceinline__ int find_item(const uint32_t *base, int n, uint32_t x)
{
    int lo = 0, hi = n - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(base + mid) <= x)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// Walks a grid-stride range over the concatenated per-item ranges given by
// `base`, calling fn(item, local_index); the item is looked up only when the
// index leaves the previous item's range.
template <class Fn>
__device__ __forceinline__ void for_each_in_items(const BatchDev *b, const uint32_t *base, uint32_t total, Fn &&fn)
{
    int item = -1;
    uint32_t lo = 0, hi = 0;
    const int n = b->n_items;
    for (uint32_t g = blockIdx.x * blockDim.x + threadIdx.x; g < total; g += gridDim.x * blockDim.x) {
        if (g < lo || g >= hi) {
            item = find_item(base, n, g);
            lo = __ldg(base + item);
            hi = __ldg(base + item + 1);
        }
        fn(item, g - lo);
    }
}

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

__global__ void __launch_bounds__(256) k_clear(const BatchDev *b)
{
    for_each_in_items(b, b->px_base, b->total_px,
                      [&](int item, uint32_t i) { b->items[item].key[i] = kEmptyKey; });
}

// world_to_camera_or_frustum (vertex_shaders.hpp:35-52): view, projection
// (rows 0-2), x and y divided by |z'|; also clears the visibility flag.
__global__ void __launch_bounds__(256) k_vertex(const BatchDev *b)
{
    for_each_in_items(b, b->vtx_base, b->total_vtx, [&](int item, uint32_t g) {
        const ItemDev &it = b->items[item];
        const float4 w = it.s.wpos[g];
        V3 p = transform3(mk3(w.x, w.y, w.z), it.v.view);
        p = transform3(p, it.v.proj);
        if (p.z != 0.0f) {
            p.x = p.x / fabsf(p.z);
            p.y = p.y / fabsf(p.z);
        }
        it.ndc[g] = make_float4(p.x, p.y, p.z, 0.0f);
        it.yes[g] = 0;
    });
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
__global__ void __launch_bounds__(256) k_flags(const BatchDev *b)
{
    for_each_in_items(b, b->tri_base, b->total_tri, [&](int item, uint32_t t) {
        const ItemDev &it = b->items[item];
        const uint4 tri = it.s.tris[t];
        const V3 a = ld3(it.ndc, tri.x), c1 = ld3(it.ndc, tri.y), c2 = ld3(it.ndc, tri.z);
        if (!inside_frustum(a, c1, c2))
            return;
        const int m = it.s.prims[tri.w].material;
        const int ds = (m >= 0 && m < it.s.n_mats) ? it.s.mats[m].double_sided : 0;
        if (ds || cross_n_z(sub3(c1, a), sub3(c2, a)) > 0.0f) {
            it.yes[tri.x] = 1;
            it.yes[tri.y] = 1;
            it.yes[tri.z] = 1;
        }
    });
}

// frustum_to_viewport (viewport.cpp:123-129) of a flagged vertex
__device__ __forceinline__ V3 load_vp(const ItemDev &it, uint32_t g)
{
    const float4 n = it.ndc[g];
    return mk3(it.v.vm00 * n.x + it.v.vm03, it.v.vm11 * n.y + it.v.vm13, n.z);
}

// Rows of fill_triangle_2's scanline range from the three screen y values:
// ceil(max y) - ceil(min y) (renderer.cpp:390-394).  The compaction uses it to
// class triangles, and the shade kernel to know which triangles had every
// span binned; both evaluate it the same way.
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
// one list, each block's entries grouped by row class so that a warp of the
// walk gets triangles of similar size; triangles crossing the near plane go to
// their own list.  One global atomic per list per block.
constexpr int kCompactBlock = 512;
__global__ void __launch_bounds__(kCompactBlock) k_compact(const BatchDev *b)
{
    __shared__ uint32_t cnt[kClasses + 1], cls_off[kClasses], base[2];
    const int lane = threadIdx.x & 31;
    int item = -1;
    uint32_t lo = 0, hi = 0;
    const uint32_t total = b->total_tri;
    // every thread of the block runs the same number of iterations (barriers inside)
    const uint32_t span = gridDim.x * blockDim.x;
    for (uint32_t g0 = blockIdx.x * blockDim.x; g0 < total; g0 += span) {
        if (threadIdx.x < kClasses + 1)
            cnt[threadIdx.x] = 0;
        __syncthreads();
        const uint32_t g = g0 + threadIdx.x;
        int list = -1;
        uint32_t t = 0;
        if (g < total) {
            if (g < lo || g >= hi) {
                item = find_item(b->tri_base, b->n_items, g);
                lo = __ldg(b->tri_base + item);
                hi = __ldg(b->tri_base + item + 1);
            }
            t = g - lo;
            const ItemDev &it = b->items[item];
            const uint4 tri = it.s.tris[t];
            if (it.yes[tri.x] && it.yes[tri.y] && it.yes[tri.z]) {
                const float4 a = it.ndc[tri.x], c1 = it.ndc[tri.y], c2 = it.ndc[tri.z];
                // fill_triangle's cases (renderer.cpp:281-318): the smallest z' decides
                if (below_near(a.z) || below_near(c1.z) || below_near(c2.z))
                    list = kClasses;
                else
                    list = row_class(row_extent(it.v.vm11 * a.y + it.v.vm13, it.v.vm11 * c1.y + it.v.vm13,
                                                it.v.vm11 * c2.y + it.v.vm13));
            }
        }
        uint32_t pos = 0;
#pragma unroll
        for (int k = 0; k <= kClasses; k++) {
            const unsigned m = __ballot_sync(0xFFFFFFFFu, list == k);
            if (!m)
                continue;
            uint32_t wb = 0;
            if (lane == 0)
                wb = atomicAdd(&cnt[k], (uint32_t)__popc(m));
            wb = __shfl_sync(0xFFFFFFFFu, wb, 0);
            if (list == k)
                pos = wb + __popc(m & ((1u << lane) - 1u));
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            uint32_t run = 0;
            for (int k = 0; k < kClasses; k++) {
                cls_off[k] = run;
                run += cnt[k];
            }
            uint32_t *c32 = reinterpret_cast<uint32_t *>(b->counters);
            base[0] = run ? atomicAdd(&c32[C_LIST], run) : 0u;
            base[1] = cnt[kClasses] ? atomicAdd(&c32[C_CLIP], cnt[kClasses]) : 0u;
        }
        __syncthreads();
        if (list == kClasses) {
            const uint32_t j = base[1] + pos;
            if (j < b->clip_cap)
                b->clip[b->clip_cap - 1 - j] = make_uint2(t, (uint32_t)item); // filled from the end
        } else if (list >= 0) {
            const uint32_t j = base[0] + cls_off[list] + pos;
            if (j < b->list_cap)
                b->list[j] = make_uint2(t, (uint32_t)item | ((uint32_t)list << 24));
        }
        __syncthreads();
    }
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

__device__ __forceinline__ uint32_t *counter32(const BatchDev *b, int w)
{
    return reinterpret_cast<uint32_t *>(b->counters) + w;
}

// Bin a long span: the qpixel state after its displacement to x1.
__device__ __forceinline__ bool bin_span(const BatchDev *b, uint32_t item, uint32_t slot, int y, int x1, int x2,
                                         const Side &Ls, const Side &Rs, uint32_t bits)
{
    const uint32_t i = atomicAdd(counter32(b, C_SPANS), 1u);
    if (i >= b->span_cap) {
        atomicExch(counter32(b, C_OVERFLOW), 1u);
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
    r.item = item;
    b->spans[i] = r;
    return true;
}

struct DepthVisitor {
    const BatchDev *b;
    const ItemDev *it;
    uint32_t item;
    uint32_t slot;
    int inline_span;
    bool bin_all; // tall triangle: every span goes to the bins
    unsigned long long drawn_n, fragments;

    __device__ __forceinline__ bool active() const { return true; }
    __device__ __forceinline__ void drawn()
    {
        drawn_n++;
        if (b->slot_flags)
            b->slot_flags[slot] = 1;
    }
    __device__ __forceinline__ void span(int y, int x1, int x2, const Side &Ls, const Side &Rs, uint32_t bits)
    {
        fragments += (unsigned long long)(x2 - x1);
        if ((bin_all || x2 - x1 > inline_span) && bin_span(b, item, slot, y, x1, x2, Ls, Rs, bits))
            return;
        const ViewDev &v = it->v;
        unsigned long long *row = it->key + ((long long)(y - v.y) * v.w - v.x);
        const uint32_t sl = slot;
        auto op = [&](int x, float z, float) {
            atomicMin(row + x, make_key(z, sl)); // result unused: a reduction, no round trip
        };
        span_pixels(x1, x2, Ls, Rs, op);
    }
};

// Records the winner's progress values (the overflow fallback and the
// near-clip triangles, whose winners the shade kernel does not replay).
struct WinnerVisitor {
    const ItemDev *it;
    uint32_t slot;
    int inline_span;
    bool all_spans; // bins overflowed: record every span here

    __device__ __forceinline__ bool active() const { return true; }
    __device__ __forceinline__ void drawn() {}
    __device__ __forceinline__ void span(int y, int x1, int x2, const Side &Ls, const Side &Rs, uint32_t bits)
    {
        if (x2 - x1 > inline_span && !all_spans)
            return; // recorded by the winner span kernel from the bins
        const ViewDev &v = it->v;
        const long long base = (long long)(y - v.y) * v.w - v.x;
        const unsigned long long *row = it->key + base;
        float4 *rec = it->prec + base;
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
// values the reference had there: the edge progress of the row and the qpixel
// progress after (tx - x1) steps (renderer.cpp:474-493).  Spans wider than
// the inline limit were recorded by the span kernels instead (use_prec).
struct ReplayVisitor {
    int tx, ty;
    int inline_span;
    bool found, use_prec;
    float4 rec;

    __device__ __forceinline__ bool active() const { return !found && !use_prec; }
    __device__ __forceinline__ void drawn() {}
    __device__ __forceinline__ void span(int y, int x1, int x2, const Side &Ls, const Side &Rs, uint32_t bits)
    {
        if (y != ty || tx < x1 || tx >= x2)
            return;
        if (x2 - x1 > inline_span) {
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

// Per-item counters of a warp: lanes grouped by item, one atomic per group.
__device__ __forceinline__ void item_add(unsigned long long *dst, uint32_t item, unsigned long long v, bool valid)
{
    const unsigned act = __ballot_sync(0xFFFFFFFFu, valid);
    if (!valid)
        return;
    const unsigned grp = __match_any_sync(act, item);
    unsigned long long sum = 0;
    for (unsigned m = grp; m; m &= m - 1)
        sum += __shfl_sync(grp, v, __ffs(m) - 1);
    if ((threadIdx.x & 31) == __ffs(grp) - 1 && sum)
        atomicAdd(dst + 2 * (size_t)item, sum);
}

__device__ __forceinline__ void warp_add(unsigned long long *dst, unsigned long long v)
{
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_down_sync(0xFFFFFFFFu, v, o);
    if ((threadIdx.x & 31) == 0 && v)
        atomicAdd(dst, v);
}

// Depth walk of the drawable triangles wholly in front of the near plane:
// fill_triangle's normal case (renderer.cpp:281-285), one sub-triangle, slot 2t.
__global__ void __launch_bounds__(128, 8) k_walk(const BatchDev *b)
{
    const uint32_t n_raw = *counter32(b, C_LIST);
    const uint32_t n = n_raw < b->list_cap ? n_raw : b->list_cap;
    unsigned long long drawn_all = 0, frags_all = 0;
    for (uint32_t i0 = blockIdx.x * blockDim.x; i0 < n; i0 += gridDim.x * blockDim.x) {
        const uint32_t i = i0 + threadIdx.x;
        DepthVisitor vis{b, nullptr, 0u, 0u, b->inline_span, false, 0ull, 0ull};
        const bool valid = i < n;
        if (valid) {
            const uint2 e = b->list[i];
            vis.item = e.y & 0xFFFFFFu;
            vis.it = &b->items[vis.item];
            vis.bin_all = (e.y >> 24) == (uint32_t)(kClasses - 1);
            const uint4 tri = vis.it->s.tris[e.x];
            V3 a = load_vp(*vis.it, tri.x), c1 = load_vp(*vis.it, tri.y), c2 = load_vp(*vis.it, tri.z);
            int pa = 0, pb = 1, pc = 2;
            sort_z_desc(a, c1, c2, pa, pb, pc);
            vis.slot = 2 * e.x;
            walk_sub(vis.it->v, a, c1, c2, vis);
        }
        item_add(b->item_counters, vis.item, vis.drawn_n, valid);
        item_add(b->item_counters + 1, vis.item, vis.fragments, valid);
        drawn_all += vis.drawn_n;
        frags_all += vis.fragments;
    }
    warp_add(&b->counters[C_DRAWN], drawn_all);
    warp_add(&b->counters[C_FRAGMENTS], frags_all);
}

// Winner records of every simple triangle's spans: runs only when the bins
// overflowed (the shade kernel replays winners otherwise).
__global__ void __launch_bounds__(128, 8) k_walk_winner(const BatchDev *b)
{
    if (!*counter32(b, C_OVERFLOW))
        return;
    const uint32_t n_raw = *counter32(b, C_LIST);
    const uint32_t n = n_raw < b->list_cap ? n_raw : b->list_cap;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint2 e = b->list[i];
        const ItemDev &it = b->items[e.y & 0xFFFFFFu];
        WinnerVisitor vis{&it, 2 * e.x, b->inline_span, true};
        const uint4 tri = it.s.tris[e.x];
        V3 a = load_vp(it, tri.x), c1 = load_vp(it, tri.y), c2 = load_vp(it, tri.z);
        int pa = 0, pb = 1, pc = 2;
        sort_z_desc(a, c1, c2, pa, pb, pc);
        walk_sub(it.v, a, c1, c2, vis);
    }
}

// ------------------------------------------------------------- near clip --

// A vertex with everything fill_triangle's clip branches need (mesh_vertex_t,
// swegl/data/model.hpp:20-29).
struct TV {
    V3 vp;     // v_viewport: screen x, y and z'
    V3 world;  // v_world
    V3 normal; // object-space normal
    V3 nworld; // normal_world
    V2 uv;
};

__device__ __forceinline__ void load_tv(const ItemDev &it, uint32_t g, TV &o)
{
    o.vp = load_vp(it, g);
    const float4 w = it.s.wpos[g];
    o.world = mk3(w.x, w.y, w.z);
    const float4 nv = it.s.nrm_v[g];
    o.normal = mk3(nv.x, nv.y, nv.z);
    const float2 uv = it.s.uv[g];
    o.uv = mk2(uv.x, uv.y);
    const float4 nw = it.s.wnrm[g];
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
__device__ __forceinline__ void clip_triangle(const ItemDev &it, uint32_t t, Emit &emit)
{
    const uint4 tri = it.s.tris[t];
    TV tv[3];
    load_tv(it, tri.x, tv[0]);
    load_tv(it, tri.y, tv[1]);
    load_tv(it, tri.z, tv[2]);
    const float *rs = it.s.node_rs + 16 * it.s.prims[tri.w].node;
    const ViewDev &v = it.v;
    const TV *a = &tv[0], *b = &tv[1], *c = &tv[2], *tp;
    bool ffv = cross_n_z(sub3(b->vp, a->vp), sub3(c->vp, a->vp)) < 0.0f;
    bool inverted_order = false;
    if (b->vp.z > a->vp.z) { tp = a; a = b; b = tp; inverted_order = !inverted_order; }
    if (c->vp.z > b->vp.z) { tp = b; b = c; c = tp; inverted_order = !inverted_order; }
    if (b->vp.z > a->vp.z) { tp = a; a = b; b = tp; inverted_order = !inverted_order; }
    const V3 v0 = a->vp, v1 = b->vp, v2 = c->vp;
    if (at_or_past_near(v2.z)) {
        emit(2 * t, *a, *b, *c, ffv); // not reached: compaction sent it to the main list
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
__global__ void __launch_bounds__(128) k_walk_clip(const BatchDev *b)
{
    const uint32_t n_raw = *counter32(b, C_CLIP);
    const uint32_t n = n_raw < b->clip_cap ? n_raw : b->clip_cap;
    const bool overflow = *counter32(b, C_OVERFLOW) != 0u;
    unsigned long long drawn_all = 0, frags_all = 0;
    for (uint32_t i0 = blockIdx.x * blockDim.x; i0 < n; i0 += gridDim.x * blockDim.x) {
        const uint32_t i = i0 + threadIdx.x;
        const bool valid = i < n;
        DepthVisitor dvis{b, nullptr, 0u, 0u, b->inline_span, false, 0ull, 0ull};
        if (valid) {
            const uint2 e = b->clip[b->clip_cap - 1 - i];
            const ItemDev &it = b->items[e.y];
            dvis.item = e.y;
            dvis.it = &it;
            WinnerVisitor wvis{&it, 0u, b->inline_span, overflow};
            auto emit = [&](uint32_t slot, const TV &a, const TV &c1, const TV &c2, bool) {
                if (!WINNER) {
                    dvis.slot = slot;
                    walk_sub(it.v, a.vp, c1.vp, c2.vp, dvis);
                } else {
                    wvis.slot = slot;
                    walk_sub(it.v, a.vp, c1.vp, c2.vp, wvis);
                }
            };
            clip_triangle(it, e.x, emit);
        }
        if (!WINNER) {
            item_add(b->item_counters, dvis.item, dvis.drawn_n, valid);
            item_add(b->item_counters + 1, dvis.item, dvis.fragments, valid);
            drawn_all += dvis.drawn_n;
            frags_all += dvis.fragments;
        }
    }
    if (!WINNER) {
        warp_add(&b->counters[C_DRAWN], drawn_all);
        warp_add(&b->counters[C_FRAGMENTS], frags_all);
    }
}

// ------------------------------------------------------------- long spans --

// Binned spans, one warp each.  The qpixel chain (top += tstep, bottom +=
// bstep per pixel, interpolator.hpp:96-100) is serial in floating point, so
// every lane runs the same 32 steps and keeps the state of its own pixel; the
// divisions, depth and key work then run on all lanes.
template <int WINNER>
__global__ void __launch_bounds__(256) k_spans(const BatchDev *b)
{
    const uint32_t n_raw = *counter32(b, C_SPANS);
    const uint32_t n = n_raw < b->span_cap ? n_raw : b->span_cap;
    if (WINNER && *counter32(b, C_OVERFLOW))
        return; // the overflow winner walk records every span
    const int lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t n_warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t i = warp; i < n; i += n_warps) {
        const SpanRec r = b->spans[i];
        const ItemDev &it = b->items[r.item];
        const int y = (int)(r.y_bits & kYMask);
        const long long base = (long long)(y - it.v.y) * it.v.w - it.v.x;
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
            unsigned long long *kp = it.key + base + x;
            if (!WINNER)
                atomicMin(kp, key);
            else if (*kp == key)
                it.prec[base + x] = make_float4(alpha, r.progL, r.progR, __uint_as_float(r.y_bits & ~kYMask));
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
// winner's progress values (renderer.cpp:433-493)
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

// One pixel (x, y relative to the viewport) of item `item`: the background of
// viewport_t::clear (viewport.cpp:88-113) or the colour of the winning
// fragment, and its depth.  Winners of near-clipped triangles are passed on
// to k_shade_clip.
__device__ __forceinline__ void shade_pixel(const BatchDev *b, uint32_t item, const ItemDev &it, int x, int y)
{
    const ViewDev &v = it.v;
    const uint32_t i = (uint32_t)y * (uint32_t)v.w + (uint32_t)x;
    const unsigned long long k = it.key[i];
    uint32_t *px = it.pixels + (long long)y * it.pitch_px + x;
    if (k == kEmptyKey) {
        *px = 0u;
        if (it.zbuf)
            it.zbuf[i] = __uint_as_float(kMaxZBits);
        return;
    }
    if (it.zbuf)
        it.zbuf[i] = __uint_as_float((uint32_t)(k >> 32));
    const uint32_t slot = (uint32_t)k;
    const uint4 tri = it.s.tris[slot >> 1];
    V3 a = load_vp(it, tri.x), c1 = load_vp(it, tri.y), c2 = load_vp(it, tri.z);
    if (below_near(a.z) || below_near(c1.z) || below_near(c2.z)) {
        const uint32_t j = atomicAdd(counter32(b, C_CLIPPX), 1u);
        if (j < b->clippx_cap)
            b->clippx[j] = make_uint2(i, item);
        return;
    }
    // fill_triangle: front_face_visible, then the z sort; fill_triangle_2: the y sort
    const bool ffv = cross_n_z(sub3(c1, a), sub3(c2, a)) < 0.0f;
    int pa = 0, pb = 1, pc = 2;
    sort_z_desc(a, c1, c2, pa, pb, pc);
    float4 rec;
    if (*counter32(b, C_OVERFLOW) || row_extent(a.y, c1.y, c2.y) > kTallRows) {
        rec = it.prec[i]; // recorded by the span kernels (or the overflow winner walk)
    } else {
        ReplayVisitor rv{x + v.x, y + v.y, b->inline_span, false, false, make_float4(0.f, 0.f, 0.f, 0.f)};
        walk_sub(v, a, c1, c2, rv);
        rec = rv.found ? rv.rec : it.prec[i];
    }
    sort_y_asc(a, c1, c2, pa, pb, pc);
    const uint32_t g0 = pa == 0 ? tri.x : (pa == 1 ? tri.y : tri.z);
    const uint32_t g1 = pb == 0 ? tri.x : (pb == 1 ? tri.y : tri.z);
    const uint32_t g2 = pc == 0 ? tri.x : (pc == 1 ? tri.y : tri.z);
    Shader sh;
    bind_material(it.s, tri.w, sh);
    const float4 w0 = it.s.wpos[g0], w1 = it.s.wpos[g1], w2 = it.s.wpos[g2];
    const float4 n0 = it.s.wnrm[g0], n1 = it.s.wnrm[g1], n2 = it.s.wnrm[g2];
    const float2 u0 = it.s.uv[g0], u1 = it.s.uv[g1], u2 = it.s.uv[g2];
    const V3 sw[3] = {mk3(w0.x, w0.y, w0.z), mk3(w1.x, w1.y, w1.z), mk3(w2.x, w2.y, w2.z)};
    const V3 sn[3] = {mk3(n0.x, n0.y, n0.z), mk3(n1.x, n1.y, n1.z), mk3(n2.x, n2.y, n2.z)};
    const V2 su[3] = {mk2(u0.x, u0.y), mk2(u1.x, u1.y), mk2(u2.x, u2.y)};
    sh_prepare_triangle(sh, sw, sn, su, !ffv);
    *px = shade_winner(sh, *it.s.lights, v, rec);
}

// Square tiles of TILE x TILE pixels, one block of TILE*TILE threads per tile.
template <int TILE>
__global__ void __launch_bounds__(TILE *TILE) k_shade(const BatchDev *b)
{
    int item = -1;
    uint32_t lo = 0, hi = 0;
    for (uint32_t tg = blockIdx.x; tg < b->total_tiles; tg += gridDim.x) {
        if (tg < lo || tg >= hi) {
            item = find_item(b->tile_base, b->n_items, tg);
            lo = __ldg(b->tile_base + item);
            hi = __ldg(b->tile_base + item + 1);
        }
        const ItemDev &it = b->items[item];
        const uint32_t tl = tg - lo;
        const int tx = (int)(tl % (uint32_t)it.tiles_x), ty = (int)(tl / (uint32_t)it.tiles_x);
        const int x = tx * TILE + (int)(threadIdx.x % TILE), y = ty * TILE + (int)(threadIdx.x / TILE);
        if (x < it.v.w && y < it.v.h)
            shade_pixel(b, (uint32_t)item, it, x, y);
    }
}

// Winners that belong to near-clipped triangles: the clip vertices are rebuilt
// exactly as fill_triangle makes them; the progress values were recorded by
// the near-clip winner walk.
__global__ void __launch_bounds__(128) k_shade_clip(const BatchDev *b)
{
    const uint32_t n_raw = *counter32(b, C_CLIPPX);
    const uint32_t n = n_raw < b->clippx_cap ? n_raw : b->clippx_cap;
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        const uint2 e = b->clippx[j];
        const ItemDev &it = b->items[e.y];
        const uint32_t i = e.x;
        const int y = (int)(i / (uint32_t)it.v.w), x = (int)(i - (uint32_t)y * (uint32_t)it.v.w);
        const uint32_t slot = (uint32_t)it.key[i];
        const float4 rec = it.prec[i];
        Shader sh;
        bool done = false;
        auto emit = [&](uint32_t sl, const TV &a, const TV &c1, const TV &c2, bool ffv) {
            if (sl != slot || done)
                return;
            const TV *p0 = &a, *p1 = &c1, *p2 = &c2, *t;
            if (p1->vp.y < p0->vp.y) { t = p0; p0 = p1; p1 = t; }
            if (p2->vp.y < p1->vp.y) { t = p1; p1 = p2; p2 = t; }
            if (p1->vp.y < p0->vp.y) { t = p0; p0 = p1; p1 = t; }
            const V3 sw[3] = {p0->world, p1->world, p2->world};
            const V3 sn[3] = {p0->nworld, p1->nworld, p2->nworld};
            const V2 su[3] = {p0->uv, p1->uv, p2->uv};
            bind_material(it.s, it.s.tris[slot >> 1].w, sh);
            sh_prepare_triangle(sh, sw, sn, su, !ffv);
            done = true;
        };
        clip_triangle(it, slot >> 1, emit);
        if (done)
            it.pixels[(long long)y * it.pitch_px + x] = shade_winner(sh, *it.s.lights, it.v, rec);
    }
}

// ------------------------------------------------------------ depth of field --

__constant__ float2 c_dof_taps[SGL_DOF_TAPS];

// Depth-of-field gather (replaces post_shader_depth_box,
// swegl/render/post_shaders.hpp:51-132).  Per pixel: view-space depth from the
// z-buffer, z = (z' - P23) / P22; circle of confusion r = K*A*|z - F| / z
// pixels, clamped to [0, max]; the mean of 32 taps of the golden-angle
// pattern (sgl_dof_taps.h) at offsets roundf(r * tap), clamped to the
// viewport, with integer sums rounded half up.  Every step is exact integer
// or IEEE float arithmetic, so the CPU oracle gives the same bits.
__global__ void __launch_bounds__(256) k_dof(const BatchDev *b)
{
    for_each_in_items(b, b->px_base, b->total_px, [&](int item, uint32_t i) {
        const ItemDev &it = b->items[item];
        if (!it.dof)
            return;
        const int w = it.v.w, h = it.v.h;
        const int y = (int)(i / (uint32_t)w), x = (int)(i - (uint32_t)y * (uint32_t)w);
        const float zp = it.zbuf[i];
        const float zv = (zp - it.p23) / it.p22;
        float r = (it.dof_ka * fabsf(zv - it.dof_focus)) / zv;
        if (!(r >= 0.0f && r <= it.dof_rmax))
            r = it.dof_rmax;
        uint32_t sb = 0, sg = 0, sr = 0;
#pragma unroll 8
        for (int k = 0; k < SGL_DOF_TAPS; k++) {
            const float2 t = c_dof_taps[k];
            int sx = x + (int)roundf(r * t.x), sy = y + (int)roundf(r * t.y);
            sx = sx < 0 ? 0 : (sx >= w ? w - 1 : sx);
            sy = sy < 0 ? 0 : (sy >= h ? h - 1 : sy);
            const uint32_t c = __ldg(it.pixels + (size_t)sy * it.pitch_px + sx);
            sb += c & 0xFFu;
            sg += (c >> 8) & 0xFFu;
            sr += (c >> 16) & 0xFFu;
        }
        const uint32_t centre = it.pixels[(size_t)y * it.pitch_px + x];
        const uint32_t out = (centre & 0xFF000000u) | (((sr + 16u) / 32u) << 16) | (((sg + 16u) / 32u) << 8) |
                             ((sb + 16u) / 32u);
        it.dof_out[(size_t)y * it.dof_pitch + x] = out;
    });
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
    static const char *names[kProfKernels] = {"k_clear",  "k_vertex",       "k_flags",
                                              "k_compact", "k_walk+clip",   "k_spans",
                                              "winner records", "k_shade", "k_dof"};
    return (k >= 0 && k < kProfKernels) ? names[k] : "?";
}

// Fold the previous launch sequence's event timings into the totals.
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

// The fixed launch sequence of a batch.  Grids do not depend on the batch:
// every kernel strides over totals it reads from device memory.
// Constant tables of the current device (the depth-of-field taps); called
// before any launch or graph capture on that device.
cudaError_t init_device_constants()
{
    float2 taps[SGL_DOF_TAPS];
    for (int k = 0; k < SGL_DOF_TAPS; k++)
        taps[k] = make_float2(sgl_dof_taps[k][0], sgl_dof_taps[k][1]);
    return cudaMemcpyToSymbol(c_dof_taps, taps, sizeof taps);
}

cudaError_t launch_dof(const BatchDev *b, cudaStream_t st)
{
    k_dof<<<sm_count() * 8, 256, 0, st>>>(b);
    return cudaGetLastError();
}

cudaError_t launch_batch(const BatchDev *b, int tile, bool any_dof, cudaStream_t st, int *launches, Profiler *prof)
{
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
    int n = 0;
    mark(PK_CLEAR);
    k_clear<<<sms * 8, 256, 0, st>>>(b);
    n++;
    mark(PK_VERTEX);
    k_vertex<<<sms * 8, 256, 0, st>>>(b);
    n++;
    mark(PK_FLAGS);
    k_flags<<<sms * 8, 256, 0, st>>>(b);
    n++;
    mark(PK_COMPACT);
    k_compact<<<sms * 4, kCompactBlock, 0, st>>>(b);
    n++;
    mark(PK_DEPTH);
    k_walk<<<sms * 8, 128, 0, st>>>(b);
    k_walk_clip<0><<<sms, 128, 0, st>>>(b);
    n += 2;
    mark(PK_SPANS);
    k_spans<0><<<sms * 4, 256, 0, st>>>(b);
    n++;
    mark(PK_WINNER);
    k_spans<1><<<sms * 4, 256, 0, st>>>(b);
    k_walk_clip<1><<<sms, 128, 0, st>>>(b);
    k_walk_winner<<<sms * 8, 128, 0, st>>>(b);
    n += 3;
    mark(PK_SHADE);
    if (tile == 8)
        k_shade<8><<<sms * 16, 64, 0, st>>>(b);
    else if (tile == 32)
        k_shade<32><<<sms * 2, 1024, 0, st>>>(b);
    else
        k_shade<16><<<sms * 8, 256, 0, st>>>(b);
    k_shade_clip<<<sms, 128, 0, st>>>(b);
    n += 2;
    mark(PK_DOF);
    if (any_dof) {
        k_dof<<<sms * 8, 256, 0, st>>>(b);
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
