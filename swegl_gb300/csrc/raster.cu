// raster.cu — sm_103a kernels of the swegl render path.
//
// Every kernel works on a batch of views (items: scene, camera, buffers) and
// is a persistent grid-stride kernel with a fixed grid that reads the batch
// totals from device memory, so one launch sequence (and one CUDA graph)
// serves any batch.  The plain one-frame-per-launch renderer is a batch of one.
//
//   k_vertex      world -> view -> projection, |z'| divide      (vertex_shaders.hpp:35-52)
//   k_flags       visibility flags of triangles                  (renderer.cpp:86-185)
//   k_compact     drawable triangles -> the walk list / the near-clip list
//   k_setup       per walk-list triangle: its scanline set-up (TriRec)
//   k_walk        rows of each 32 set-ups dealt across a warp's lanes,
//                 fragment keys folded with an atomic min; then the warp's
//                 share of the near-clip triangles and of the tall triangles
//   k_spans       long spans binned by the walk, one warp each
//   k_winners     winner records of binned spans and near-clip triangles
//                 (every span after a bin overflow)
//   k_shade       per pixel: background or the winner's colour, and depth;
//                 winners are queued so that shading runs on full warps
//   k_dof         depth-of-field gather of the items that ask for it
//
// Depth test.  The reference draws triangles in order and keeps a fragment
// when z < zbuffer (strict, src/render/renderer.cpp:489-499), so the earliest
// drawn of equal-depth fragments wins.  Each fragment here folds the 64-bit
// key (float bits of z << 32 | draw slot) into its pixel with atomicMin: z is
// above 0.001, so its bits order like the floats, and the draw slot
// (2 * draw-order triangle + clip sub-triangle) breaks ties in draw order.
// The shade kernel then replays the winner's row and pixel steps from the
// triangle's set-up record to recover the progress values the reference
// shaded with; spans too long to replay cheaply have them recorded by the
// span kernels instead.  The depth keys start every launch sequence empty:
// new key pools are filled once and the shade kernel empties what it reads.
#include <cstdint>

#include "sgl_cull.h"
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

// Depth-key reduction without a return value (red.global.min.u64): the
// 64-bit atomicMin() returns the old key, and a warp would wait for that round
// trip on every fragment.
__device__ __forceinline__ void key_min(unsigned long long *p, unsigned long long v)
{
    asm volatile("red.global.min.u64 [%0], %1;\n" ::"l"(p), "l"(v) : "memory");
}

// Asynchronous 4-byte global -> shared copies (cp.async), committed as groups.
__device__ __forceinline__ void cp_async4(void *smem, const void *gmem)
{
    const uint32_t sa = (uint32_t)__cvta_generic_to_shared(smem);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_async_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory"); }

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

// k_world for one posed request: the same transforms under the request's
// node matrices, into its own arrays (texture coordinates are pose-free and
// stay the scene's).
__global__ void k_pose(SceneDev s, const float *node_world, const float *node_rs, float4 *wpos, float4 *wnrm)
{
    const uint32_t g = blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= s.n_vertices)
        return;
    const uint32_t n = s.vnode[g];
    const float4 p = s.pos_u[g];
    const float4 q = s.nrm_v[g];
    const V3 w = transform3(mk3(p.x, p.y, p.z), node_world + 16 * n);
    const V3 nw = normalize3(normalize3(rotate_n(mk3(q.x, q.y, q.z), node_rs + 16 * n)));
    wpos[g] = make_float4(w.x, w.y, w.z, 0.0f);
    wnrm[g] = make_float4(nw.x, nw.y, nw.z, 0.0f);
}

// The box of each primitive's world positions (a warp per primitive), for the
// fused pass's whole-primitive frustum test: pbox[2 q] = centre, pbox[2 q + 1]
// = half extent.  NaN coordinates are left out (a triangle with one fails
// each test of inside_camera_frustum that its other vertices fail, the
// comparisons with NaN being false); a box that is empty or not finite gets a
// NaN centre and is never culled.
__global__ void k_box(SceneDev s, const float4 *wpos, float4 *pbox)
{
    const uint32_t q = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
    if (q >= s.n_prims)
        return;
    const uint4 gq = s.pgeo[q];
    V3 lo = mk3(INFINITY, INFINITY, INFINITY), hi = mk3(-INFINITY, -INFINITY, -INFINITY);
    for (uint32_t i = lane; i < gq.y; i += 32) {
        if (!in_bounds(gq.x + i < s.n_vertices, CHK_NDC, gq.x + i))
            break;
        const float4 w = wpos[gq.x + i];
        lo = mk3(fminf(lo.x, w.x), fminf(lo.y, w.y), fminf(lo.z, w.z));
        hi = mk3(fmaxf(hi.x, w.x), fmaxf(hi.y, w.y), fmaxf(hi.z, w.z));
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        lo.x = fminf(lo.x, __shfl_xor_sync(0xFFFFFFFFu, lo.x, o));
        lo.y = fminf(lo.y, __shfl_xor_sync(0xFFFFFFFFu, lo.y, o));
        lo.z = fminf(lo.z, __shfl_xor_sync(0xFFFFFFFFu, lo.z, o));
        hi.x = fmaxf(hi.x, __shfl_xor_sync(0xFFFFFFFFu, hi.x, o));
        hi.y = fmaxf(hi.y, __shfl_xor_sync(0xFFFFFFFFu, hi.y, o));
        hi.z = fmaxf(hi.z, __shfl_xor_sync(0xFFFFFFFFu, hi.z, o));
    }
    if (lane == 0) {
        float4 c, h;
        cull_box(make_float3(lo.x, lo.y, lo.z), make_float3(hi.x, hi.y, hi.z), c, h);
        pbox[2 * q] = c;
        pbox[2 * q + 1] = h;
    }
}

// world_to_camera_or_frustum (vertex_shaders.hpp:35-52): view, projection
// (rows 0-2), x and y divided by |z'|; also clears the visibility flag.  The
// item's matrices stay in registers while the index is inside it.  Each
// thread takes kGeomPer vertices (a warp 32 * kGeomPer consecutive ones) and
// issues their loads first.
constexpr int kGeomPer = 4;
__global__ void __launch_bounds__(256) k_vertex(const BatchDev *b)
{
    uint32_t lo = 0, hi = 0;
    float m[24];
    const float4 *wpos = nullptr;
    float4 *ndc = nullptr;
    uint8_t *yes = nullptr;
    const uint8_t *vsmall = nullptr; // a mixed scene: vertices the fused pass transforms
    const uint32_t total = b->total_gvtx;
    auto bind = [&](uint32_t g) {
        const int item = find_item(b->g_vtx_base, b->n_items, g);
        lo = __ldg(b->g_vtx_base + item);
        hi = __ldg(b->g_vtx_base + item + 1);
        const ItemDev &it = b->items[item];
#pragma unroll
        for (int k = 0; k < 12; k++) {
            m[k] = it.v.view[k];
            m[12 + k] = it.v.proj[k];
        }
        wpos = it.s.wpos;
        ndc = it.ndc;
        yes = it.yes;
        vsmall = it.s.vsmall;
    };
    auto project = [&](uint32_t l, float4 w) {
        if (vsmall && vsmall[l])
            return;
        V3 p = transform3(mk3(w.x, w.y, w.z), m);
        p = transform3(p, m + 12);
        if (p.z != 0.0f) {
            p.x = p.x / fabsf(p.z);
            p.y = p.y / fabsf(p.z);
        }
        if (!in_bounds(l < hi - lo, CHK_NDC, l))
            return;
        ndc[l] = make_float4(p.x, p.y, p.z, 0.0f);
        yes[l] = below_near(p.z) ? kYesBehind : 0; // kYesDrawn is set by k_flags
    };
    // a warp takes 32 * kGeomPer consecutive vertices, lane + 32 u each
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t stride = gridDim.x * blockDim.x * kGeomPer;
    for (uint32_t g0 = ((blockIdx.x * blockDim.x + threadIdx.x) & ~31u) * kGeomPer + lane; g0 < total; g0 += stride) {
        const uint32_t glast = g0 + 32 * (kGeomPer - 1);
        if (g0 < lo || g0 >= hi)
            bind(g0);
        if (glast < hi && glast < total) {
            const uint32_t l = g0 - lo;
            float4 w[kGeomPer];
#pragma unroll
            for (int u = 0; u < kGeomPer; u++)
                w[u] = wpos[l + 32 * u];
#pragma unroll
            for (int u = 0; u < kGeomPer; u++)
                project(l + 32 * u, w[u]);
        } else {
            for (uint32_t g = g0; g <= glast && g < total; g += 32) {
                if (g < lo || g >= hi)
                    bind(g);
                project(g - lo, wpos[g - lo]);
            }
        }
    }
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
constexpr int kFlagsPer = 2;
__global__ void __launch_bounds__(256) k_flags(const BatchDev *b)
{
    uint32_t lo = 0, hi = 0;
    const uint4 *tris = nullptr;
    const float4 *ndc = nullptr;
    uint8_t *yes = nullptr;
    const PrimDesc *prims = nullptr;
    const MatDesc *mats = nullptr;
    const uint8_t *psmall = nullptr; // a mixed scene: primitives of the fused pass
    int n_mats = 0;
    const uint32_t total = b->total_gtri;
    auto bind = [&](uint32_t g) {
        const int item = find_item(b->g_tri_base, b->n_items, g);
        lo = __ldg(b->g_tri_base + item);
        hi = __ldg(b->g_tri_base + item + 1);
        const ItemDev &it = b->items[item];
        tris = it.s.tris;
        ndc = it.ndc;
        yes = it.yes;
        prims = it.s.prims;
        mats = it.s.mats;
        n_mats = it.s.n_mats;
        psmall = it.s.psmall;
    };
    auto flag = [&](uint4 tri, V3 a, V3 c1, V3 c2) {
        if ((psmall && psmall[tri.w]) || !inside_frustum(a, c1, c2))
            return;
        // front facing, else double sided (the material is read only then)
        bool vis = cross_z_positive(sub3(c1, a), sub3(c2, a));
        if (!vis) {
            const int m = prims[tri.w].material;
            vis = m >= 0 && m < n_mats && mats[m].double_sided;
        }
        if (vis) {
            yes[tri.x] = kYesDrawn | (below_near(a.z) ? kYesBehind : 0);
            yes[tri.y] = kYesDrawn | (below_near(c1.z) ? kYesBehind : 0);
            yes[tri.z] = kYesDrawn | (below_near(c2.z) ? kYesBehind : 0);
        }
    };
    // a warp takes 32 * kFlagsPer consecutive triangles, lane + 32 u each,
    // and issues all their loads before the tests
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t stride = gridDim.x * blockDim.x * kFlagsPer;
    for (uint32_t g0 = ((blockIdx.x * blockDim.x + threadIdx.x) & ~31u) * kFlagsPer + lane; g0 < total; g0 += stride) {
        const uint32_t glast = g0 + 32 * (kFlagsPer - 1);
        if (g0 < lo || g0 >= hi)
            bind(g0);
        if (glast < hi && glast < total) {
            const uint32_t l = g0 - lo;
            uint4 t[kFlagsPer];
#pragma unroll
            for (int u = 0; u < kFlagsPer; u++)
                t[u] = tris[l + 32 * u];
            V3 a[kFlagsPer], c1[kFlagsPer], c2[kFlagsPer];
#pragma unroll
            for (int u = 0; u < kFlagsPer; u++) {
                a[u] = ld3(ndc, t[u].x);
                c1[u] = ld3(ndc, t[u].y);
                c2[u] = ld3(ndc, t[u].z);
            }
#pragma unroll
            for (int u = 0; u < kFlagsPer; u++)
                flag(t[u], a[u], c1[u], c2[u]);
        } else {
            for (uint32_t g = g0; g <= glast && g < total; g += 32) {
                if (g < lo || g >= hi)
                    bind(g);
                const uint4 tri = tris[g - lo];
                flag(tri, ld3(ndc, tri.x), ld3(ndc, tri.y), ld3(ndc, tri.z));
            }
        }
    }
}

// frustum_to_viewport (viewport.cpp:123-129) of a flagged vertex
__device__ __forceinline__ V3 load_vp(const ItemDev &it, uint32_t g)
{
    const float4 n = it.ndc[g];
    return mk3(it.v.vm00 * n.x + it.v.vm03, it.v.vm11 * n.y + it.v.vm13, n.z);
}

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

// Per-item counters (drawn triangles, fragments) of a warp, summed in
// registers while all of the warp's lanes work on one item and added to the
// item's counters when the item changes (one atomic per counter then); an
// iteration whose lanes span several items adds per item at once.  Every
// lane of the warp calls add() and flush().
struct ItemAcc {
    uint32_t item = 0xFFFFFFFFu;
    unsigned long long v0 = 0, v1 = 0;

    __device__ __forceinline__ void flush(const BatchDev *b)
    {
        if (item != 0xFFFFFFFFu) {
            warp_add(b->item_counters + 2 * (size_t)item, v0);
            warp_add(b->item_counters + 2 * (size_t)item + 1, v1);
        }
        item = 0xFFFFFFFFu;
        v0 = v1 = 0;
    }
    __device__ __forceinline__ void add(const BatchDev *b, uint32_t it, unsigned long long a0, unsigned long long a1,
                                        bool valid)
    {
        const unsigned act = __ballot_sync(0xFFFFFFFFu, valid);
        if (!act)
            return;
        const uint32_t first = __shfl_sync(0xFFFFFFFFu, it, __ffs(act) - 1);
        if (__all_sync(0xFFFFFFFFu, !valid || it == first)) {
            if (first != item) {
                flush(b);
                item = first;
            }
            if (valid) {
                v0 += a0;
                v1 += a1;
            }
        } else {
            item_add(b->item_counters, it, a0, valid);
            item_add(b->item_counters + 1, it, a1, valid);
        }
    }
};

// The record slot of a near-clipped batch triangle: flags = kRecClip.
__device__ __forceinline__ void mark_clip(const BatchDev *b, uint32_t r)
{
    if (in_bounds(r < b->list_cap, CHK_REC, r))
        reinterpret_cast<uint32_t *>(b->recs + r)[kRecFlagsWord] = kRecClip;
}

// 32-bit batch counter w (C_*)
__device__ __forceinline__ uint32_t *counter32(const BatchDev *b, int w)
{
    return reinterpret_cast<uint32_t *>(b->counters) + w;
}

// Reserve n0 walk-list and n1 clip-list entries with one atomic: the two
// 32-bit counters C_LIST and C_CLIP are the halves of one 64-bit counter word
// (a list holds fewer than 2^31 entries, so the low half never carries).
// Returns the previous values (C_LIST low, C_CLIP high).
static_assert(C_LIST % 2 == 0 && C_CLIP == C_LIST + 1, "list counters share a 64-bit word");
__device__ __forceinline__ unsigned long long reserve_lists(const BatchDev *b, uint32_t n0, uint32_t n1)
{
    if (!(n0 | n1))
        return 0ull;
    return atomicAdd(b->counters + C_LIST / 2, ((unsigned long long)n1 << 32) | n0);
}

// Drawable triangles (all three vertices flagged, renderer.cpp:248-253) into
// the walk list; triangles crossing the near plane go to their own list and
// are marked in the record map.  One global atomic per list per block.
constexpr int kCompactBlock = 512;
__global__ void __launch_bounds__(kCompactBlock) k_compact(const BatchDev *b)
{
    __shared__ uint32_t cnt[2], base[2];
    const int lane = threadIdx.x & 31;
    int item = -1;
    uint32_t lo = 0, hi = 0;
    const uint4 *tris = nullptr;
    const uint8_t *yes = nullptr;
    const uint8_t *psmall = nullptr; // a mixed scene: primitives of the fused pass
    const uint32_t total = b->total_gtri;
    ItemAcc acc; // triangles counted as drawn here (no pixel column)
    // every thread of the block runs the same number of iterations (barriers inside)
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t g0 = blockIdx.x * blockDim.x; g0 < total; g0 += stride) {
        if (threadIdx.x < 2)
            cnt[threadIdx.x] = 0;
        __syncthreads();
        const uint32_t g = g0 + threadIdx.x;
        int list = -1;
        bool xsliver = false;
        uint32_t t = 0;
        if (g < total) {
            if (g < lo || g >= hi) {
                item = find_item(b->g_tri_base, b->n_items, g);
                lo = __ldg(b->g_tri_base + item);
                hi = __ldg(b->g_tri_base + item + 1);
                const ItemDev &it = b->items[item];
                tris = it.s.tris;
                yes = it.yes;
                psmall = it.s.psmall;
            }
            t = g - lo;
            const uint4 tri = tris[t];
            const bool general = !psmall || !psmall[tri.w];
            const uint32_t ya = general ? yes[tri.x] : 0u, yb = general ? yes[tri.y] : 0u,
                           yc = general ? yes[tri.z] : 0u;
            if (ya & yb & yc & kYesDrawn) {
                // fill_triangle's cases (renderer.cpp:281-318): the smallest z' decides
                list = ((ya | yb | yc) & kYesBehind) ? 1 : 0;
                if (list == 0) {
                    const ItemDev &it = b->items[item];
                    const float y0 = it.v.vm11 * it.ndc[tri.x].y + it.v.vm13;
                    const float y1 = it.v.vm11 * it.ndc[tri.y].y + it.v.vm13;
                    const float y2 = it.v.vm11 * it.ndc[tri.z].y + it.v.vm13;
                    const float lo_y = fminf(y0, fminf(y1, y2)), hi_y = fmaxf(y0, fmaxf(y1, y2));
                    // (finite or infinite y only: with a NaN the set-up's sort decides)
                    if (y0 == y0 && y1 == y1 && y2 == y2) {
                        if (f2i(ceilf(lo_y)) == f2i(ceilf(hi_y))) {
                            // fill_triangle_2 draws nothing when its first and last
                            // rows coincide (ceil of the smallest and largest y,
                            // renderer.cpp:389-391): such a triangle never reaches
                            // the set-up or the walk, and is not counted
                            list = -1;
                        } else {
                            // No pixel column either: every row's span [ceil(xl),
                            // ceil(xr)) is empty when the triangle's x range, widened
                            // by the walk's rounding, holds no integer boundary.  The
                            // walked edge positions are the exact ones (inside the
                            // range) up to the start's rounding and one rounding per
                            // row step, (rows + 17) u (max |x| + eps) in all (u =
                            // 2^-24); eps is over twice that.  Such a triangle reached
                            // the set-up in the reference, so it is counted as drawn,
                            // but it covers no pixel and gets no set-up record.
                            const float x0 = it.v.vm00 * it.ndc[tri.x].x + it.v.vm03;
                            const float x1 = it.v.vm00 * it.ndc[tri.y].x + it.v.vm03;
                            const float x2 = it.v.vm00 * it.ndc[tri.z].x + it.v.vm03;
                            const float mx = fmaxf(fabsf(x0), fmaxf(fabsf(x1), fabsf(x2)));
                            const float rows = ceilf(hi_y) - ceilf(lo_y);
                            const float eps = (rows + 32.0f) * 0x1p-23f * (mx + 1.0f);
                            const float lo_x = fminf(x0, fminf(x1, x2)) - eps;
                            const float hi_x = fmaxf(x0, fmaxf(x1, x2)) + eps;
                            if (ceilf(lo_x) == ceilf(hi_x)) {
                                list = -1;
                                xsliver = true;
                                if (b->slot_flags)
                                    b->slot_flags[2 * t] = 1;
                            }
                        }
                    }
                }
            }
        }
        acc.add(b, (uint32_t)item, 1ull, 0ull, xsliver);
        uint32_t pos = 0;
#pragma unroll
        for (int k = 0; k < 2; k++) {
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
            const unsigned long long old = reserve_lists(b, cnt[0], cnt[1]);
            base[0] = (uint32_t)old;
            base[1] = (uint32_t)(old >> 32);
        }
        __syncthreads();
        if (list == 1) {
            const uint32_t j = base[1] + pos;
            if (j < b->clip_cap)
                b->clip[b->clip_cap - 1 - j] = make_uint2(t, (uint32_t)item); // filled from the end
            mark_clip(b, __ldg(b->tri_base + item) + t);
        } else if (list == 0) {
            const uint32_t j = base[0] + pos;
            if (j < b->list_cap)
                b->list[j] = make_uint2(__ldg(b->tri_base + item) + t, (uint32_t)item);
        }
        __syncthreads();
    }
    acc.flush(b);
}

// The geometry of fused scenes (every primitive within kFuseVerts vertices
// and kFuseTris triangles): one warp per primitive runs k_vertex, k_flags and
// k_compact on it with the vertex positions and flags in shared memory.  A
// primitive owns its vertices (no two vertex ranges overlap), so its
// triangles are the only ones that flag them (renderer.cpp:86-185 flags a
// node's primitives before any is drawn, and each primitive's vertices are
// its own), and its compaction needs nothing from other warps.
//
// Items are taken in groups that read the same vertex data (the views of one
// scene in the batch; the reference likewise transforms a scene to world
// space once for all the viewports of a render call, renderer.hpp:27-34).
// A block takes a chunk of kGeomWarps consecutive primitives of a group and
// runs each warp's primitive for every item of the group: the primitive's
// first 64 triangles stay in registers as local vertex indices and its world
// positions are read again per item (from L1 after the first).  The items go
// in passes of kGeomPass: per item the warp records its walk-list and
// clip-list decisions as ballot masks, and after the pass one global atomic
// reserves both lists for all the pass's items and warps (reserve_lists).
constexpr int kGeomPass = 8;            // items per list reservation
constexpr int kGeomTG = kFuseTris / 32; // groups of 32 triangles
constexpr int kGeomBlocks = 4;          // resident blocks per SM the pass is compiled for
struct GeomShared {
    float pos[kGeomWarps][3 * kFuseVerts];         // x, y, z' of each vertex (for the item in hand)
    uint8_t yes[kGeomWarps][kFuseVerts];
    uint32_t walk[kGeomPass][kGeomWarps][kGeomTG]; // per 32 triangles: ballot of the walk list
    uint32_t clip[kGeomPass][kGeomWarps][kGeomTG]; // ... of the clip list
    uint32_t cnt[kGeomPass][kGeomWarps][2];        // entries of each list, then their first positions
    uint32_t nx[kGeomPass][kGeomWarps];            // drawable triangles without a pixel column
    float view[kGeomWarps][28];                    // the warp's copy of the item in hand: view and
                                                   // projection rows 0-2, vm00, vm03, vm11, vm13
};
static_assert(kFuseVerts <= 256, "local vertex indices are bytes");
constexpr size_t kGeomSmem = sizeof(GeomShared);

// The local vertex indices of triangle t of a fused primitive (a | b << 8 | c << 16).
__device__ __forceinline__ uint32_t geom_tri(const uint4 *tris, uint4 gq, uint32_t t)
{
    const uint4 tri = tris[gq.z + t];
    in_bounds(tri.x - gq.x < gq.y && tri.y - gq.x < gq.y && tri.z - gq.x < gq.y, CHK_LOCAL, gq.z + t);
    return (tri.x - gq.x) | ((tri.y - gq.x) << 8) | ((tri.z - gq.x) << 16);
}

// Bit i (i < n <= 8) set when item grp_items[v0 + i] sees none of the
// triangles of primitive q (box pbox[2 q], pbox[2 q + 1]): the box is in the
// region z' > 0 and in one beyond a side plane (ViewDev::cull).  Lane 4 i + r
// tests item i's side r; the mask is the same in every lane.  A box with a
// NaN is in no region.
__device__ __forceinline__ uint32_t geom_unseen(const BatchDev *b, const float4 *pbox, uint32_t q, uint32_t v0,
                                                uint32_t n, uint32_t lane)
{
    bool out = false;
    if ((lane >> 2) < n) {
        const float4 *cull = &b->items[__ldg(b->grp_items + v0 + (lane >> 2))].v.cull[0][0];
        const float4 bc = pbox[2 * q], bh = pbox[2 * q + 1];
        const float4 ba = make_float4(fabsf(bc.x) + bh.x, fabsf(bc.y) + bh.y, fabsf(bc.z) + bh.z, 0.0f);
        out = cull_region(cull + 2 * (lane & 3), bc, bh, ba) < 0.0f && cull_region(cull + 8, bc, bh, ba) < 0.0f;
    }
    const unsigned m = __ballot_sync(0xFFFFFFFFu, out);
    uint32_t u = 0;
#pragma unroll
    for (int i = 0; i < kGeomPass; i++)
        u |= ((m >> (4 * i)) & 15u) ? 1u << i : 0u;
    return u;
}

__global__ void __launch_bounds__(kGeomWarps * 32, kGeomBlocks) k_geom(const BatchDev *b)
{
    extern __shared__ __align__(16) unsigned char geom_smem[];
    GeomShared &S = *reinterpret_cast<GeomShared *>(geom_smem);
    const int warp = threadIdx.x >> 5;
    const uint32_t lane = threadIdx.x & 31;
    const unsigned below = (1u << lane) - 1u;
    float *pos = S.pos[warp];
    uint8_t *sy = S.yes[warp];
    float *vw = S.view[warp];
    int g = -1;
    uint32_t c_lo = 0, c_hi = 0;
    const uint32_t total = b->total_chunks;
    // every thread of the block runs the same iterations (barriers inside)
    for (uint32_t c = blockIdx.x; c < total; c += gridDim.x) {
        if (c < c_lo || c >= c_hi) {
            g = find_item(b->grp_chunk_base, b->n_groups, c);
            c_lo = __ldg(b->grp_chunk_base + g);
            c_hi = __ldg(b->grp_chunk_base + g + 1);
        }
        const uint32_t i_lo = __ldg(b->grp_item_base + g), i_hi = __ldg(b->grp_item_base + g + 1);
        const SceneDev &sc = b->items[__ldg(b->grp_items + i_lo)].s; // vertex data shared by the group
        const uint32_t q = (c - c_lo) * kGeomWarps + warp;             // this warp's primitive
        const bool has = q < sc.n_prims && (!sc.psmall || sc.psmall[q]); // (a mixed scene's larger ones: general passes)
        uint4 gq = make_uint4(0u, 0u, 0u, 0u); // first vertex, vertex count, first triangle, triangle count
        bool ds = false;
        uint32_t tr0 = 0, tr1 = 0; // the first 64 triangles, local vertex indices
        uint32_t unseen = 0; // bit vi: item vi of the pass in hand sees none of the primitive
        const float4 *wpos = sc.wpos;
        const uint4 *tris = sc.tris;
        if (has) {
            gq = sc.pgeo[q];
            gq.y = min(gq.y, kFuseVerts); // (a fused scene's primitives are within both limits)
            gq.w = min(gq.w, kFuseTris);
            if (lane < gq.w)
                tr0 = geom_tri(tris, gq, lane);
            if (lane + 32 < gq.w)
                tr1 = geom_tri(tris, gq, lane + 32);
            ds = sc.pshade[q].double_sided != 0;
        }
        for (uint32_t v0 = i_lo; v0 < i_hi; v0 += kGeomPass) {
            const int nv = (int)min((uint32_t)kGeomPass, i_hi - v0);
            if (has && sc.pbox)
                unseen = geom_unseen(b, sc.pbox, q, v0, (uint32_t)nv, lane);
            for (int vi = 0; vi < nv; vi++) {
                uint32_t c0 = 0, c1 = 0, nx = 0;
                const bool seen = has && !((unseen >> vi) & 1u);
                if (!seen && has) {
                    // the item sees none of the primitive's triangles
                    if (lane < (uint32_t)kGeomTG) {
                        S.walk[vi][warp][lane] = 0u;
                        S.clip[vi][warp][lane] = 0u;
                    }
                }
                if (seen) {
                    const uint32_t item = __ldg(b->grp_items + v0 + vi);
                    const ItemDev &it = b->items[item];
                    __syncwarp(); // the previous item's reads of pos, sy and vw are done
                    if (lane < 12) {
                        vw[lane] = it.v.view[lane];
                        vw[12 + lane] = it.v.proj[lane];
                    } else if (lane == 12) {
                        vw[24] = it.v.vm00;
                        vw[25] = it.v.vm03;
                        vw[26] = it.v.vm11;
                        vw[27] = it.v.vm13;
                    }
                    float4 *ndc = it.ndc + gq.x;
                    __syncwarp();
                    // world_to_camera_or_frustum (vertex_shaders.hpp:35-52), as
                    // k_vertex; 128 vertices per round, their loads issued first
                    for (uint32_t i0 = 0; i0 < gq.y; i0 += 128) {
                        float4 w[4];
#pragma unroll
                        for (int k = 0; k < 4; k++)
                            if (i0 + lane + 32 * k < gq.y)
                                w[k] = wpos[gq.x + i0 + lane + 32 * k];
#pragma unroll
                        for (int k = 0; k < 4; k++) {
                            const uint32_t i = i0 + lane + 32 * k;
                            if (i < gq.y) {
                                V3 v = transform3(mk3(w[k].x, w[k].y, w[k].z), vw);
                                v = transform3(v, vw + 12);
                                if (v.z != 0.0f) {
                                    v.x = v.x / fabsf(v.z);
                                    v.y = v.y / fabsf(v.z);
                                }
                                if (in_bounds(gq.x + i < sc.n_vertices, CHK_NDC, gq.x + i))
                                    ndc[i] = make_float4(v.x, v.y, v.z, 0.0f);
                                pos[3 * i] = v.x;
                                pos[3 * i + 1] = v.y;
                                pos[3 * i + 2] = v.z;
                                sy[i] = below_near(v.z) ? kYesBehind : 0;
                            }
                        }
                    }
                    __syncwarp();
                    // visibility flags (renderer.cpp:86-185), as k_flags; every
                    // store to a vertex writes the same value
                    for (uint32_t t = lane; t < gq.w; t += 32) {
                        const uint32_t tp = t < 32 ? tr0 : (t < 64 ? tr1 : geom_tri(tris, gq, t));
                        const uint32_t ia = tp & 0xFFu, ib = (tp >> 8) & 0xFFu, ic = tp >> 16;
                        const V3 a = mk3(pos[3 * ia], pos[3 * ia + 1], pos[3 * ia + 2]);
                        const V3 c1v = mk3(pos[3 * ib], pos[3 * ib + 1], pos[3 * ib + 2]);
                        const V3 c2v = mk3(pos[3 * ic], pos[3 * ic + 1], pos[3 * ic + 2]);
                        if (inside_frustum(a, c1v, c2v) && (ds || cross_z_positive(sub3(c1v, a), sub3(c2v, a)))) {
                            sy[ia] = kYesDrawn | (below_near(a.z) ? kYesBehind : 0);
                            sy[ib] = kYesDrawn | (below_near(c1v.z) ? kYesBehind : 0);
                            sy[ic] = kYesDrawn | (below_near(c2v.z) ? kYesBehind : 0);
                        }
                    }
                    __syncwarp();
                    // the compaction's decisions, as k_compact
                    const float vm00 = vw[24], vm03 = vw[25], vm11 = vw[26], vm13 = vw[27];
                    for (uint32_t t0 = 0; t0 < gq.w; t0 += 32) {
                        const uint32_t t = t0 + lane;
                        int d = 0; // 0 none, 1 walk list, 2 clip list, 3 no pixel column
                        if (t < gq.w) {
                            const uint32_t tp = t < 32 ? tr0 : (t < 64 ? tr1 : geom_tri(tris, gq, t));
                            const uint32_t ia = tp & 0xFFu, ib = (tp >> 8) & 0xFFu, ic = tp >> 16;
                            const uint32_t ya = sy[ia], yb = sy[ib], yc = sy[ic];
                            if (ya & yb & yc & kYesDrawn) {
                                if ((ya | yb | yc) & kYesBehind) {
                                    d = 2;
                                } else {
                                    d = 1;
                                    const float y0 = vm11 * pos[3 * ia + 1] + vm13;
                                    const float y1 = vm11 * pos[3 * ib + 1] + vm13;
                                    const float y2 = vm11 * pos[3 * ic + 1] + vm13;
                                    const float lo_y = fminf(y0, fminf(y1, y2)), hi_y = fmaxf(y0, fmaxf(y1, y2));
                                    if (y0 == y0 && y1 == y1 && y2 == y2) {
                                        if (f2i(ceilf(lo_y)) == f2i(ceilf(hi_y))) {
                                            d = 0; // no row
                                        } else {
                                            const float x0 = vm00 * pos[3 * ia] + vm03;
                                            const float x1 = vm00 * pos[3 * ib] + vm03;
                                            const float x2 = vm00 * pos[3 * ic] + vm03;
                                            const float mx = fmaxf(fabsf(x0), fmaxf(fabsf(x1), fabsf(x2)));
                                            const float rows = ceilf(hi_y) - ceilf(lo_y);
                                            const float eps = (rows + 32.0f) * 0x1p-23f * (mx + 1.0f);
                                            const float lo_x = fminf(x0, fminf(x1, x2)) - eps;
                                            const float hi_x = fmaxf(x0, fmaxf(x1, x2)) + eps;
                                            if (ceilf(lo_x) == ceilf(hi_x)) {
                                                d = 3; // no pixel column
                                                if (b->slot_flags)
                                                    b->slot_flags[2 * (gq.z + t)] = 1;
                                            }
                                        }
                                    }
                                }
                            }
                        }
                        const unsigned m1 = __ballot_sync(0xFFFFFFFFu, d == 1);
                        const unsigned m2 = __ballot_sync(0xFFFFFFFFu, d == 2);
                        const unsigned m3 = __ballot_sync(0xFFFFFFFFu, d == 3);
                        if (lane == 0) {
                            S.walk[vi][warp][t0 >> 5] = m1;
                            S.clip[vi][warp][t0 >> 5] = m2;
                        }
                        c0 += __popc(m1);
                        c1 += __popc(m2);
                        nx += __popc(m3);
                    }
                }
                if (lane == 0) {
                    S.cnt[vi][warp][0] = c0;
                    S.cnt[vi][warp][1] = c1;
                    S.nx[vi][warp] = nx;
                }
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                // first positions per item and warp, one reservation for the pass
                uint32_t n0 = 0, n1 = 0;
                for (int vi = 0; vi < nv; vi++) {
                    uint32_t x = 0;
                    for (int w = 0; w < kGeomWarps; w++) {
                        const uint32_t a0 = S.cnt[vi][w][0], a1 = S.cnt[vi][w][1];
                        S.cnt[vi][w][0] = n0;
                        S.cnt[vi][w][1] = n1;
                        n0 += a0;
                        n1 += a1;
                        x += S.nx[vi][w];
                    }
                    // triangles counted as drawn here: they reached fill_triangle_2's set-up
                    if (x)
                        atomicAdd(b->item_counters + 2 * (size_t)__ldg(b->grp_items + v0 + vi), (unsigned long long)x);
                }
                const unsigned long long old = reserve_lists(b, n0, n1);
                const uint32_t g0 = (uint32_t)old, g1 = (uint32_t)(old >> 32);
                for (int vi = 0; vi < nv; vi++)
                    for (int w = 0; w < kGeomWarps; w++) {
                        S.cnt[vi][w][0] += g0;
                        S.cnt[vi][w][1] += g1;
                    }
            }
            __syncthreads();
            if (has) {
                for (int vi = 0; vi < nv; vi++) {
                    uint32_t o0 = S.cnt[vi][warp][0], o1 = S.cnt[vi][warp][1];
                    const uint32_t item = __ldg(b->grp_items + v0 + vi);
                    const uint32_t tlo = __ldg(b->tri_base + item);
                    for (uint32_t t0 = 0; t0 < gq.w; t0 += 32) {
                        const unsigned m1 = S.walk[vi][warp][t0 >> 5], m2 = S.clip[vi][warp][t0 >> 5];
                        const uint32_t t = t0 + lane;
                        if ((m1 >> lane) & 1u) {
                            const uint32_t j = o0 + __popc(m1 & below);
                            if (j < b->list_cap)
                                b->list[j] = make_uint2(tlo + gq.z + t, item);
                        } else if ((m2 >> lane) & 1u) {
                            const uint32_t j = o1 + __popc(m2 & below);
                            if (j < b->clip_cap)
                                b->clip[b->clip_cap - 1 - j] = make_uint2(gq.z + t, item); // from the end
                            mark_clip(b, tlo + gq.z + t);
                        }
                        o0 += __popc(m1);
                        o1 += __popc(m2);
                    }
                }
            }
            __syncthreads(); // the counts and masks are rewritten by the next pass
        }
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
            if (in_bounds(x >= v.x && x < v.x + v.w && y >= v.y && y < v.y + v.h, CHK_KEY,
                          (unsigned long long)(uint32_t)y << 32 | (uint32_t)x))
                key_min(row + x, make_key(z, sl));
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

// ------------------------------------------------------- row-parallel walk --
//
// The walk of fill_triangle_2 is serial only along its edges: row k needs the
// edges after k steps (x += ratio, top += tstep, bottom += bstep, renderer.cpp
// :553-556), and each span needs the qpixel chain from its left end.  The
// steps are float additions, so any thread can reach row k by repeating them
// from the set-up; the divisions of a row (edge progress, span set-up) and of
// its pixels then run wherever that row is.  A warp takes 32 triangles, each
// lane makes its triangle's set-up (the TriRec), and the warp's rows are
// dealt out across the lanes.  Triangles with more than kTallRows rows are
// walked by the whole warp, 32 rows at a time, and every one of their spans
// goes to the long-span kernels.

constexpr int kWalkWarps = 4;
#ifndef SGL_WALK_MIN_BLOCKS
#define SGL_WALK_MIN_BLOCKS 6 // resident blocks per SM the walk is compiled for (caps its registers)
#endif
// Per-warp shared copy of the lanes' set-ups, sm[field][lane]: fields 0-31 are
// the words of TriRec in order, so the warp can store whole records; the row
// is padded to 33 words so that both the per-lane and the per-record accesses
// are free of bank conflicts.
enum {
    F_LX, F_LT, F_LB, F_LR, F_LTS, F_LBS, // long edge: x, top, bottom, ratio, tstep, bstep
    F_UX, F_UT, F_UB, F_UR, F_UTS, F_UBS, // upper short edge
    F_DX, F_DT, F_DB, F_DR, F_DTS, F_DBS, // lower short edge
    F_Z0, F_Z1, F_Z2, F_YS, F_YL, F_NU, F_ND, F_FLAGS, F_SLOT, F_ITEM, F_G0, F_G1, F_G2, F_PRIM,
    F_FRAGS, // fragments of the lane's triangle (shared atomics of the lanes walking its rows)
    F_INCL,  // inclusive prefix of the rows dealt out, per lane
    kWalkFields
};
constexpr int kWalkPitch = 33;
static_assert(F_PRIM == 31 && sizeof(TriRec) == 32 * sizeof(uint32_t), "shared set-up fields follow TriRec");

// interpolator_g<1>::InitSelf then DisplaceStartingPoint (interpolator.hpp:
// 60-84), with 1/z1 and 1/z2 passed in (the same divisions, made once per
// vertex).  The progress of the displaced state is not formed here: every
// reader divides top by bottom itself, as step() would have.
__device__ __forceinline__ void edge_init(float dist, float rz1, float rz2, float move, float &top, float &bot,
                                          float &ts, float &bs)
{
    const float alphastep = 1.0f / dist;
    bot = rz1;
    top = 0.0f;
    top = top * bot;
    ts = (1.0f * rz2 - top) * alphastep;
    bs = (rz2 - bot) * alphastep;
    top = top + ts * move;
    bot = bot + bs * move;
}

// The inputs of one walked row: both edges at the half's first row with
// their constants, the steps to take, the row and its span bits.
struct RowIn {
    float lx, lt, lb, lr, lts, lbs, lz, ldv; // long edge; value() = lz + ldv * progress
    float sx, st, sb, sr, sts, sbs, sz, sdv; // short edge of the row's half
    int y, ls, ss;
    bool llr;
    uint32_t bits;
};

// Row k of a set-up (k < n_u: upper half): `lg` is the long edge (x, top,
// bottom, ratio, tstep, bstep), `sh` the short edge of the row's half.
__device__ __forceinline__ void row_in(RowIn &r, int k, const float lg[6], const float sh[6], float z0, float z1,
                                       float z2, int y_s, int y_l, int n_u, uint32_t flags)
{
    r.lx = lg[0]; r.lt = lg[1]; r.lb = lg[2]; r.lr = lg[3]; r.lts = lg[4]; r.lbs = lg[5];
    r.sx = sh[0]; r.st = sh[1]; r.sb = sh[2]; r.sr = sh[3]; r.sts = sh[4]; r.sbs = sh[5];
    r.lz = z0;
    r.ldv = z2 - z0;
    r.ls = k;
    if (k < n_u) {
        r.sz = z0;
        r.sdv = z1 - z0;
        r.y = y_s + k;
        r.ss = k;
        r.llr = (flags & kRecLLRUpper) != 0u;
        r.bits = r.llr ? kBitLLR : 0u;
    } else {
        r.sz = z1;
        r.sdv = z2 - z1;
        r.y = y_l + (k - n_u);
        r.ss = k - n_u;
        r.llr = (flags & kRecLLRLower) != 0u;
        r.bits = kBitLower | (r.llr ? kBitLLR : 0u);
    }
}

// A row after its steps: the span [x1, x2) clipped to the viewport
// (renderer.cpp:466-472) and the left and right edge (Ls, Rs).
struct RowSpan {
    int x1, x2;
    float Lx, Lt, Lb, Lz, Ldv, Rx, Rt, Rb, Rz, Rdv;
};

__device__ __forceinline__ void row_span(RowIn &r, int vx, int vw, RowSpan &o)
{
    for (int k = 0; k < r.ls; k++) {
        r.lx = r.lx + r.lr;
        r.lt = r.lt + r.lts;
        r.lb = r.lb + r.lbs;
    }
    for (int k = 0; k < r.ss; k++) {
        r.sx = r.sx + r.sr;
        r.st = r.st + r.sts;
        r.sb = r.sb + r.sbs;
    }
    if (r.llr) {
        o.Lx = r.sx; o.Lt = r.st; o.Lb = r.sb; o.Lz = r.sz; o.Ldv = r.sdv;
        o.Rx = r.lx; o.Rt = r.lt; o.Rb = r.lb; o.Rz = r.lz; o.Rdv = r.ldv;
    } else {
        o.Lx = r.lx; o.Lt = r.lt; o.Lb = r.lb; o.Lz = r.lz; o.Ldv = r.ldv;
        o.Rx = r.sx; o.Rt = r.st; o.Rb = r.sb; o.Rz = r.sz; o.Rdv = r.sdv;
    }
    o.x1 = f2i(ceilf(o.Lx));
    if (o.x1 < vx)
        o.x1 = vx;
    o.x2 = f2i(ceilf(o.Rx));
    if (o.x2 > vx + vw)
        o.x2 = vx + vw;
}

// The qpixel interpolator of a span after its displacement to x1, and the
// progress of both edges (renderer.cpp:474-480, prepare_for_scanline).  With
// `steps` > 0 the interpolator is also stepped that many pixels: top and
// bottom take every addition of the reference's per-pixel steps, and alpha,
// which each step recomputes from them alone, is divided out once at the end
// (the same value as the last step's).
__device__ __forceinline__ void span_interp(const RowSpan &o, Interp &q, float &pl, float &pr, int steps = 0)
{
    pl = o.Lt / o.Lb;
    pr = o.Rt / o.Rb;
    q.init_self(o.Rx - o.Lx, o.Lz + o.Ldv * pl, o.Rz + o.Rdv * pr);
    const float move = (float)o.x1 - o.Lx;
    q.top = q.top + q.tstep * move; // Interp::displace without its division
    q.bottom = q.bottom + q.bstep * move;
    for (int k = 0; k < steps; k++) {
        q.top = q.top + q.tstep;
        q.bottom = q.bottom + q.bstep;
    }
    q.alpha = q.top / q.bottom;
}

// Bins the spans of the lanes that ask for it (one atomic per warp).  Every
// lane of the warp calls it; returns whether this lane's span was binned.
__device__ __forceinline__ bool bin_span_warp(const BatchDev *b, bool want, uint32_t item, uint32_t slot, int y,
                                              const RowSpan &o, const Interp &q, float pl, float pr, uint32_t bits)
{
    const unsigned m = __ballot_sync(0xFFFFFFFFu, want);
    if (!m)
        return false;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(m) - 1;
    uint32_t base = 0;
    if (lane == leader)
        base = atomicAdd(counter32(b, C_SPANS), (uint32_t)__popc(m));
    base = __shfl_sync(0xFFFFFFFFu, base, leader);
    if (!want)
        return false;
    const uint32_t i = base + __popc(m & ((1u << lane) - 1u));
    if (i >= b->span_cap) {
        atomicExch(counter32(b, C_OVERFLOW), 1u);
        return false;
    }
    SpanRec r;
    r.slot = slot;
    r.y_bits = (uint32_t)y | bits;
    r.x1 = o.x1;
    r.x2 = o.x2;
    r.top = q.top;
    r.tstep = q.tstep;
    r.bottom = q.bottom;
    r.bstep = q.bstep;
    r.v0 = q.v0;
    r.dv = q.dv;
    r.progL = pl;
    r.progR = pr;
    r.item = item;
    b->spans[i] = r;
    return true;
}

// One span's pixels into the depth keys (the opaque branch of
// fill_half_triangle, renderer.cpp:484-499, as a key reduction).
// The view fields the walk needs, kept in registers while the item stays.
struct WalkView {
    uint32_t item;
    int x, y, w, h;
    unsigned long long *key;
    int inline_span;
    __device__ __forceinline__ void load(const BatchDev *b, uint32_t i)
    {
        const ItemDev &it = b->items[i];
        item = i;
        x = it.v.x;
        y = it.v.y;
        w = it.v.w;
        h = it.v.h;
        key = it.key;
    }
};

__device__ __forceinline__ void span_depth(const WalkView &v, int y, uint32_t slot, int x1, int x2, Interp q)
{
    unsigned long long *row = v.key + ((long long)(y - v.y) * v.w - v.x);
    for (int x = x1; x < x2; x++, q.step()) {
        const float z = q.value();
        if (below_near(z) || __float_as_uint(z) >= kMaxZBits)
            continue;
        if (in_bounds(x >= v.x && x < v.x + v.w && y >= v.y && y < v.y + v.h, CHK_KEY,
                      (unsigned long long)(uint32_t)y << 32 | (uint32_t)x))
            key_min(row + x, make_key(z, slot));
    }
}

// Fragment capture of a view with transparency layers (a layered batch has
// one item): the pool counter and its per-pixel chains.
__device__ __forceinline__ unsigned long long *frag_counter(const BatchDev *b)
{
    return b->counters + C_FRAGS / 2;
}

// One span's fragments stored from pool entry `at` on, each with its view
// pixel in the `next` field (k_link chains them afterwards); pixels skipped
// at the near plane are stored as holes (kFragEnd).
__device__ __forceinline__ void span_frags(const BatchDev *b, uint32_t row_px, uint32_t slot, int x1, int x2,
                                           Interp q, float pl, float pr, uint32_t bits, uint32_t at)
{
    Frag *pool = b->frags;
    const float fb = __uint_as_float(bits);
    for (int x = x1; x < x2; x++, q.step()) {
        const float z = q.value();
        const bool keep = !below_near(z) && __float_as_uint(z) < kMaxZBits;
        const uint32_t k = at + (uint32_t)(x - x1);
        reinterpret_cast<float4 *>(pool + k)[0] = make_float4(q.alpha, pl, pr, fb);
        reinterpret_cast<uint4 *>(pool + k)[1] =
            make_uint4(__float_as_uint(z), slot, keep ? row_px + (uint32_t)x : kFragEnd, 0u);
    }
}

typedef uint32_t WalkRow[kWalkPitch];

__device__ __forceinline__ float smf(const WalkRow *S, int f, int o) { return __uint_as_float(S[f][o]); }

__device__ __forceinline__ void smem_row_in(RowIn &r, const WalkRow *S, int o, int k)
{
    const int n_u = (int)S[F_NU][o];
    const int sf = k < n_u ? F_UX : F_DX;
    float lg[6], sh[6];
#pragma unroll
    for (int f = 0; f < 6; f++) {
        lg[f] = smf(S, F_LX + f, o);
        sh[f] = smf(S, sf + f, o);
    }
    row_in(r, k, lg, sh, smf(S, F_Z0, o), smf(S, F_Z1, o), smf(S, F_Z2, o), (int)S[F_YS][o], (int)S[F_YL][o], n_u,
           S[F_FLAGS][o]);
}

// Set-up of triangle t of `item` (list entry i): fill_triangle's z sort
// (renderer.cpp:264-279), fill_triangle_2's y sort, edges and halves
// (:375-460), into the TriRec of batch triangle r (t = r - tri_base[item]).
// Returns whether the triangle reached scanline set-up (y0 != y2); the record
// of one that did not has no rows.
__device__ __forceinline__ bool tri_setup(const BatchDev *b, uint32_t r, uint32_t item, bool &tall)
{
    tall = false;
    const uint32_t t = r - __ldg(b->tri_base + item);
    const ItemDev &it = b->items[item];
    const ViewDev &v = it.v;
    const uint4 tri = it.s.tris[t];
    V3 a = load_vp(it, tri.x), c1 = load_vp(it, tri.y), c2 = load_vp(it, tri.z);
    const bool ffv = cross_z_negative(sub3(c1, a), sub3(c2, a));
    int pa = 0, pb = 1, pc = 2;
    sort_z_desc(a, c1, c2, pa, pb, pc);
    sort_y_asc(a, c1, c2, pa, pb, pc);
    const V3 v0 = a, v1 = c1, v2 = c2;
    const int y0 = f2i(ceilf(v0.y)), y1 = f2i(ceilf(v1.y)), y2 = f2i(ceilf(v2.y));
    if (!in_bounds(r < b->list_cap, CHK_REC, r))
        return false;
    float4 *dst = reinterpret_cast<float4 *>(b->recs + r);
    if (y0 == y2) {
        // no rows: n_u = n_d = 0
        dst[5] = make_float4(0.0f, 0.0f, 0.0f, __int_as_float(0));
        dst[6] = make_float4(__int_as_float(0), 0.0f, 0.0f, __uint_as_float(item));
        return false;
    }
    const uint32_t slot = 2 * t;
    if (b->slot_flags)
        b->slot_flags[slot] = 1;
    const float rz0 = 1.0f / v0.z, rz1 = 1.0f / v1.z, rz2 = 1.0f / v2.z;
    const int ys = y0 < v.y ? v.y : y0;
    float ltop, lbot, lts, lbs;
    const float lmove = (float)ys - v0.y;
    const float lratio = (v2.x - v0.x) / (v2.y - v0.y);
    edge_init(v2.y - v0.y, rz0, rz2, lmove, ltop, lbot, lts, lbs);
    const float lx = v0.x + lratio * lmove;
    uint32_t flags = ffv ? kRecFFV : 0u;
    int n_u = 0, n_d = 0, y_l = 0;
    float ux = 0.0f, utop = 0.0f, ubot = 0.0f, uratio = 0.0f, uts = 0.0f, ubs = 0.0f;
    float dx = 0.0f, dtop = 0.0f, dbot = 0.0f, dratio = 0.0f, dts = 0.0f, dbs = 0.0f;
    if (y1 >= v.y) {
        uratio = (v1.x - v0.x) / (v1.y - v0.y);
        const int yend = y1 < v.y + v.h ? y1 : v.y + v.h;
        edge_init(v1.y - v0.y, rz0, rz1, lmove, utop, ubot, uts, ubs);
        ux = v0.x + uratio * lmove;
        if (lratio > uratio)
            flags |= kRecLLRUpper;
        n_u = yend > ys ? yend - ys : 0;
    }
    if (y1 < v.y + v.h) {
        dratio = (v2.x - v1.x) / (v2.y - v1.y);
        const int y = y1 > v.y ? y1 : v.y;
        const int yend = y2 < v.y + v.h ? y2 : v.y + v.h;
        const float move = (float)y - v1.y;
        edge_init(v2.y - v1.y, rz1, rz2, move, dtop, dbot, dts, dbs);
        dx = v1.x + dratio * move;
        if (lratio < dratio)
            flags |= kRecLLRLower;
        y_l = y;
        n_d = yend > y ? yend - y : 0;
    }
    if (n_u + n_d > kTallRows) {
        flags |= kRecTall;
        tall = true;
    }
    const uint32_t g0 = pa == 0 ? tri.x : (pa == 1 ? tri.y : tri.z);
    const uint32_t g1 = pb == 0 ? tri.x : (pb == 1 ? tri.y : tri.z);
    const uint32_t g2 = pc == 0 ? tri.x : (pc == 1 ? tri.y : tri.z);
    dst[0] = make_float4(lx, ltop, lbot, lratio);
    dst[1] = make_float4(lts, lbs, ux, utop);
    dst[2] = make_float4(ubot, uratio, uts, ubs);
    dst[3] = make_float4(dx, dtop, dbot, dratio);
    dst[4] = make_float4(dts, dbs, v0.z, v1.z);
    dst[5] = make_float4(v2.z, __int_as_float(ys), __int_as_float(y_l), __int_as_float(n_u));
    dst[6] = make_float4(__int_as_float(n_d), __uint_as_float(flags), __uint_as_float(slot), __uint_as_float(item));
    dst[7] = make_float4(__uint_as_float(g0), __uint_as_float(g1), __uint_as_float(g2), __uint_as_float(tri.w));
    return true;
}

// Set-up of every walk list entry, one thread each.
__global__ void __launch_bounds__(256) k_setup(const BatchDev *b)
{
    const uint32_t n_raw = *counter32(b, C_LIST);
    const uint32_t n = n_raw < b->list_cap ? n_raw : b->list_cap;
    ItemAcc acc;
    const uint32_t stride = gridDim.x * blockDim.x;
    // the loop runs the same number of times on every lane of a warp
    for (uint32_t i0 = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u; i0 < n; i0 += stride) {
        const uint32_t i = i0 + (threadIdx.x & 31);
        bool drawn = false, tall = false;
        uint32_t item = 0, r = 0;
        if (i < n) {
            const uint2 e = b->list[i];
            r = e.x;
            item = e.y;
            drawn = tri_setup(b, r, item, tall);
        }
        // tall triangles are walked by a whole warp each, in k_walk_rare
        const unsigned tm = __ballot_sync(0xFFFFFFFFu, tall);
        if (tm) {
            const int lane = threadIdx.x & 31, leader = __ffs(tm) - 1;
            uint32_t tb = 0;
            if (lane == leader)
                tb = atomicAdd(counter32(b, C_TALL), (uint32_t)__popc(tm));
            tb = __shfl_sync(0xFFFFFFFFu, tb, leader);
            if (tall)
                b->tall[tb + __popc(tm & ((1u << lane) - 1u))] = r;
        }
        acc.add(b, item, drawn ? 1ull : 0ull, 0ull, i < n);
    }
    acc.flush(b);
}

// One row of triangle `slot` of `item` on this lane; every lane of the warp
// calls it (act = this lane has a row).  Spans wider than the inline limit,
// and every span of a tall triangle, go to the long-span kernels.  Returns the
// row's fragments.  `v` caches the item's view (reloaded when it changes).
// With FRAGS (a view with transparency layers) every fragment is stored
// instead: the warp reserves its lanes' fragments with one atomic per round
// of rows, and a binned span carries its first pool entry in the span
// record's `item` field.
template <bool FRAGS>
__device__ __forceinline__ int walk_row(const BatchDev *b, WalkView &v, uint32_t item, uint32_t slot, RowIn &r,
                                        bool act, bool bin_all)
{
    if (act && item != v.item)
        v.load(b, item);
    RowSpan sp;
    sp.x1 = sp.x2 = 0;
    if (act)
        row_span(r, v.x, v.w, sp);
    const bool has = act && sp.x1 < sp.x2;
    Interp q;
    float pl = 0.0f, pr = 0.0f;
    if (has)
        span_interp(sp, q, pl, pr);
    const bool want = has && (bin_all || sp.x2 - sp.x1 > v.inline_span);
    if constexpr (FRAGS) {
        const int lane = threadIdx.x & 31;
        const uint32_t n = has ? (uint32_t)(sp.x2 - sp.x1) : 0u;
        uint32_t incl = n;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t u = __shfl_up_sync(0xFFFFFFFFu, incl, d);
            if (lane >= d)
                incl += u;
        }
        unsigned long long base = 0;
        if (lane == 31 && incl)
            base = atomicAdd(frag_counter(b), (unsigned long long)incl);
        base = __shfl_sync(0xFFFFFFFFu, base, 31);
        const unsigned long long at = base + incl - n;
        const bool fits = at + n <= (unsigned long long)b->frag_cap; // else counted only: the view is redone
        if (!bin_span_warp(b, want && fits, (uint32_t)at, slot, r.y, sp, q, pl, pr, r.bits) && has && fits)
            span_frags(b, (uint32_t)((r.y - v.y) * v.w - v.x), slot, sp.x1, sp.x2, q, pl, pr, r.bits,
                       (uint32_t)at);
    } else {
        if (!bin_span_warp(b, want, item, slot, r.y, sp, q, pl, pr, r.bits) && has)
            span_depth(v, r.y, slot, sp.x1, sp.x2, q);
    }
    return has ? sp.x2 - sp.x1 : 0;
}

// A tall triangle (list entry i), walked by the whole warp: for each 32 rows
// every lane runs the 32 edge steps and keeps the state of its own row, so
// no lane repeats more than 32 steps per row it walks.  Every span is binned.
// Returns this lane's fragments.
template <bool FRAGS>
__device__ __forceinline__ uint32_t walk_tall(const BatchDev *b, uint32_t i)
{
    const int lane = threadIdx.x & 31;
    const float4 *q = reinterpret_cast<const float4 *>(b->recs + i);
    const float4 q0 = q[0], q1 = q[1], q2 = q[2], q3 = q[3], q4 = q[4], q5 = q[5], q6 = q[6];
    const float lg[6] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y};
    const float up[6] = {q1.z, q1.w, q2.x, q2.y, q2.z, q2.w};
    const float dn[6] = {q3.x, q3.y, q3.z, q3.w, q4.x, q4.y};
    const float z0 = q4.z, z1 = q4.w, z2 = q5.x;
    const int y_s = __float_as_int(q5.y), y_l = __float_as_int(q5.z), n_u = __float_as_int(q5.w);
    const int n_d = __float_as_int(q6.x);
    const uint32_t flags = __float_as_uint(q6.y), slot = __float_as_uint(q6.z), item = __float_as_uint(q6.w);
    const int n = n_u + n_d;
    uint32_t frags = 0;
    WalkView v;
    v.load(b, item);
    v.inline_span = b->inline_span;
    float lx = lg[0], lt = lg[1], lb = lg[2];
    float sx = up[0], st = up[1], sb = up[2];
    for (int r0 = 0; r0 < n; r0 += 32) {
        float mlx = 0.0f, mlt = 0.0f, mlb = 0.0f, msx = 0.0f, mst = 0.0f, msb = 0.0f;
        for (int k = 0; k < 32; k++) {
            const int rr = r0 + k;
            if (rr == n_u) { // the lower half starts on its own short edge
                sx = dn[0];
                st = dn[1];
                sb = dn[2];
            }
            if (k == lane) {
                mlx = lx; mlt = lt; mlb = lb;
                msx = sx; mst = st; msb = sb;
            }
            lx = lx + lg[3];
            lt = lt + lg[4];
            lb = lb + lg[5];
            if (rr < n_u) {
                sx = sx + up[3];
                st = st + up[4];
                sb = sb + up[5];
            } else {
                sx = sx + dn[3];
                st = st + dn[4];
                sb = sb + dn[5];
            }
        }
        const int k = r0 + lane;
        const bool act = k < n;
        RowIn r;
        row_in(r, act ? k : 0, lg, (act && k >= n_u) ? dn : up, z0, z1, z2, y_s, y_l, n_u, flags);
        r.lx = mlx; r.lt = mlt; r.lb = mlb; // already stepped to the row
        r.sx = msx; r.st = mst; r.sb = msb;
        r.ls = 0;
        r.ss = 0;
        frags += (uint32_t)walk_row<FRAGS>(b, v, item, slot, r, act, true);
    }
    return frags;
}

// the rare depth walks, defined with the near-clip code below
__device__ __noinline__ void walk_clip_depth(const BatchDev *b, ItemAcc &acc);
template <bool FRAGS>
__device__ __noinline__ void walk_tall_all(const BatchDev *b, ItemAcc &acc);

// Depth walk of the drawable triangles wholly in front of the near plane
// (fill_triangle's normal case, renderer.cpp:281-285: one sub-triangle, slot
// 2t).  Each warp takes groups of 32 list entries (warp-strided), loads their
// set-ups into shared memory (one 128-byte record per load) and deals their
// rows across its lanes.  FRAGS: the fragment capture of a layered view (the
// near-clipped triangles are captured by k_frags).
template <bool FRAGS, bool STRIDED>
__global__ void __launch_bounds__(kWalkWarps * 32, SGL_WALK_MIN_BLOCKS) k_walk(const BatchDev *b)
{
    __shared__ WalkRow sm[kWalkWarps][2][kWalkFields];
    const int lane = threadIdx.x & 31;
    const uint32_t n_raw = *counter32(b, C_LIST);
    const uint32_t n = n_raw < b->list_cap ? n_raw : b->list_cap;
    const uint32_t n_groups = (n + 31) / 32;
    // STRIDED (a batch of one view, kSeqOne): group g holds entries
    // g + j * n_groups (j < 32), so every group samples the whole list and the
    // large triangles of nearby primitives, which sit together in list order,
    // spread over all groups and warps (1080p frame: 41.7 -> 30.3 us).  In a
    // batch of several views a strided group would mix the views' triangles,
    // whose view parameters each row then reloads (serving: 5.5 -> 12.3 us
    // per request), so there group g holds entries 32 g + j.
    auto entry = [&](uint32_t g, uint32_t j) -> uint32_t { return STRIDED ? g + j * n_groups : 32 * g + j; };
    auto count = [&](uint32_t g) -> uint32_t {
        if (STRIDED)
            return min(32u, (n - g + n_groups - 1) / n_groups);
        return n - 32 * g < 32u ? n - 32 * g : 32u;
    };
    // the record (batch triangle) of entry `lane` of group g; loaded one
    // group ahead of its fetch, so that the copies do not wait for it
    auto rec_of = [&](uint32_t g) -> uint32_t {
        const uint32_t i = entry(g, (uint32_t)lane);
        return g < n_groups && i < n ? b->list[i].x : 0u;
    };
    // record j of group g -> word `lane` of field row `lane`, column j
    auto fetch = [&](uint32_t g, uint32_t rec, WalkRow *D) {
        if (g < n_groups) {
            const uint32_t cnt = count(g);
#pragma unroll 8
            for (uint32_t j = 0; j < cnt; j++) {
                const uint32_t rj = __shfl_sync(0xFFFFFFFFu, rec, j);
                if (in_bounds(rj < b->list_cap, CHK_REC, rj))
                    cp_async4(&D[lane][j], reinterpret_cast<const uint32_t *>(b->recs + rj) + lane);
            }
        }
        cp_async_commit();
    };
    ItemAcc acc;
    WalkView view;
    view.item = 0xFFFFFFFFu;
    view.inline_span = b->inline_span;
    // Warps take groups g, g + W, g + 2W, ... (W warps in the grid; work
    // queues were measured slower: 41 -> 48 us on the 1080p frame).  While
    // group g is walked, the records of the next one are copied in and the
    // list entries of the one after are loaded.
    const uint32_t W = (gridDim.x * blockDim.x) >> 5;
    uint32_t g = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    uint32_t g_next = g + W;
    int buf = 0;
    fetch(g, rec_of(g), sm[threadIdx.x >> 5][0]);
    uint32_t rec_next = rec_of(g_next);
    while (g < n_groups) {
        fetch(g_next, rec_next, sm[threadIdx.x >> 5][buf ^ 1]);
        const uint32_t g_after = g_next + W;
        rec_next = rec_of(g_after);
        cp_async_wait<1>(); // this group's copies are done
        WalkRow *S = sm[threadIdx.x >> 5][buf];
        const uint32_t cnt = count(g);
        S[F_FRAGS][lane] = 0;
        __syncwarp();
        const bool valid = (uint32_t)lane < cnt;
        const int n_u = valid ? (int)S[F_NU][lane] : 0, n_d = valid ? (int)S[F_ND][lane] : 0;
        const bool tall = valid && (S[F_FLAGS][lane] & kRecTall) != 0u; // walked by k_walk_rare
        // rows of the non-tall triangles, dealt across the lanes
        int incl = tall ? 0 : n_u + n_d;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const int u = __shfl_up_sync(0xFFFFFFFFu, incl, d);
            if (lane >= d)
                incl += u;
        }
        S[F_INCL][lane] = (uint32_t)incl;
        __syncwarp();
        const int total = (int)S[F_INCL][31];
        for (int p0 = 0; p0 < total; p0 += 32) {
            const int p = p0 + lane;
            int o = 0;
#pragma unroll
            for (int st = 16; st >= 1; st >>= 1)
                if ((int)S[F_INCL][o + st - 1] <= p)
                    o += st;
            o = o > 31 ? 31 : o;
            const bool act = p < total;
            RowIn r;
            if (act) {
                const int ex = o > 0 ? (int)S[F_INCL][o - 1] : 0;
                smem_row_in(r, S, o, p - ex);
            }
            const int fr = walk_row<FRAGS>(b, view, S[F_ITEM][o], S[F_SLOT][o], r, act, false);
            if (fr)
                atomicAdd(&S[F_FRAGS][o], (uint32_t)fr);
        }
        __syncwarp();
        acc.add(b, valid ? S[F_ITEM][lane] : 0u, 0ull, valid ? (unsigned long long)S[F_FRAGS][lane] : 0ull, valid);
        __syncwarp();
        g = g_next;
        g_next = g_after;
        buf ^= 1;
    }
    cp_async_wait<0>();
    // then this warp's share of the near-clip and the tall triangles
    if (!FRAGS)
        walk_clip_depth(b, acc);
    walk_tall_all<FRAGS>(b, acc);
    acc.flush(b);
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
    bool ffv = cross_z_negative(sub3(b->vp, a->vp), sub3(c->vp, a->vp));
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
        ffv = cross_z_negative(sub3(n1.vp, v0), sub3(n2.vp, v0));
        if (inverted_order)
            ffv = !ffv;
        emit(2 * t, *a, n1, n2, ffv);
    } else {
        TV n1, n2;
        clip_vertex(v, n1, *a, *c, (v0.z - 0.001f) / (v0.z - v2.z), rs);
        clip_vertex(v, n2, *b, *c, (v1.z - 0.001f) / (v1.z - v2.z), rs);
        ffv = cross_z_negative(sub3(v1, v0), sub3(n2.vp, v0));
        if (inverted_order)
            ffv = !ffv;
        emit(2 * t, *a, *b, n2, ffv);
        ffv = cross_z_negative(sub3(n2.vp, v0), sub3(n1.vp, v0));
        if (inverted_order)
            ffv = !ffv;
        emit(2 * t + 1, *a, n2, n1, ffv);
    }
}

// Depth walk of the near-clip triangles (fill_triangle's clip cases), one
// thread each, over a warp-strided share of the clip list.  Out of line: rare,
// and its register and stack use stay off the row walk.
__device__ __noinline__ void walk_clip_depth(const BatchDev *b, ItemAcc &acc)
{
    const uint32_t n_raw = *counter32(b, C_CLIP);
    const uint32_t n = n_raw < b->clip_cap ? n_raw : b->clip_cap;
    const uint32_t lane = threadIdx.x & 31;
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, n_warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t i0 = 32 * gw; i0 < n; i0 += 32 * n_warps) {
        const uint32_t i = i0 + lane;
        const bool valid = i < n;
        DepthVisitor dvis{b, nullptr, 0u, 0u, b->inline_span, false, 0ull, 0ull};
        if (valid) {
            const uint2 e = b->clip[b->clip_cap - 1 - i];
            const ItemDev &it = b->items[e.y];
            dvis.item = e.y;
            dvis.it = &it;
            auto emit = [&](uint32_t slot, const TV &a, const TV &c1, const TV &c2, bool) {
                dvis.slot = slot;
                walk_sub(it.v, a.vp, c1.vp, c2.vp, dvis);
            };
            clip_triangle(it, e.x, emit);
        }
        acc.add(b, dvis.item, dvis.drawn_n, dvis.fragments, valid);
    }
}

// Depth walk (or fragment capture) of the tall triangles, one warp each
// (warp-strided).
template <bool FRAGS>
__device__ __noinline__ void walk_tall_all(const BatchDev *b, ItemAcc &acc)
{
    const uint32_t nt_raw = *counter32(b, C_TALL);
    const uint32_t nt = nt_raw < b->list_cap ? nt_raw : b->list_cap;
    const uint32_t gw = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, n_warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t k = gw; k < nt; k += n_warps) {
        const uint32_t i = b->tall[k];
        const uint32_t fr = walk_tall<FRAGS>(b, i);
        acc.add(b, b->recs[i].item, 0ull, fr, true);
    }
}

// Winner records of what the shade kernel does not replay, after the depth
// keys are final: binned spans (one warp each, the qpixel chain as in
// k_spans), near-clip triangles (one thread each) and, after a bin overflow,
// every span of the walk list.
__device__ __forceinline__ void spans_pass(const BatchDev *b, bool winner);

__device__ __noinline__ void winner_clip(const BatchDev *b, bool overflow)
{
    const uint32_t n_raw = *counter32(b, C_CLIP);
    const uint32_t n = n_raw < b->clip_cap ? n_raw : b->clip_cap;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint2 e = b->clip[b->clip_cap - 1 - i];
        const ItemDev &it = b->items[e.y];
        WinnerVisitor wvis{&it, 0u, b->inline_span, overflow};
        auto emit = [&](uint32_t slot, const TV &a, const TV &c1, const TV &c2, bool) {
            wvis.slot = slot;
            walk_sub(it.v, a.vp, c1.vp, c2.vp, wvis);
        };
        clip_triangle(it, e.x, emit);
    }
}

__device__ __noinline__ void winner_overflow(const BatchDev *b)
{
    const uint32_t n_raw = *counter32(b, C_LIST);
    const uint32_t n = n_raw < b->list_cap ? n_raw : b->list_cap;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const uint2 e = b->list[i];
        const ItemDev &it = b->items[e.y];
        const uint32_t t = e.x - __ldg(b->tri_base + e.y);
        WinnerVisitor vis{&it, 2 * t, b->inline_span, true};
        const uint4 tri = it.s.tris[t];
        V3 a = load_vp(it, tri.x), c1 = load_vp(it, tri.y), c2 = load_vp(it, tri.z);
        int pa = 0, pb = 1, pc = 2;
        sort_z_desc(a, c1, c2, pa, pb, pc);
        walk_sub(it.v, a, c1, c2, vis);
    }
}

__global__ void __launch_bounds__(256) k_winners(const BatchDev *b)
{
    const bool overflow = *counter32(b, C_OVERFLOW) != 0u;
    if (overflow) {
        winner_overflow(b); // records every span, the binned ones included
    } else {
        spans_pass(b, true);
    }
    winner_clip(b, overflow);
}

// ------------------------------------------------------------- long spans --

// Binned spans, one warp each.  The qpixel chain (top += tstep, bottom +=
// bstep per pixel, interpolator.hpp:96-100) is serial in floating point, so
// every lane runs the same 32 steps and keeps the state of its own pixel; the
// divisions, depth and key work then run on all lanes.
__device__ __forceinline__ void spans_pass(const BatchDev *b, bool winner)
{
    const uint32_t n_raw = *counter32(b, C_SPANS);
    const uint32_t n = n_raw < b->span_cap ? n_raw : b->span_cap;
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
            if (!in_bounds(x >= it.v.x && x < it.v.x + it.v.w && y >= it.v.y && y < it.v.y + it.v.h,
                           winner ? CHK_PREC : CHK_KEY, (unsigned long long)(uint32_t)y << 32 | (uint32_t)x))
                continue;
            if (!winner)
                key_min(kp, key);
            else if (*kp == key)
                it.prec[base + x] = make_float4(alpha, r.progL, r.progR, __uint_as_float(r.y_bits & ~kYMask));
        }
    }
}

__global__ void __launch_bounds__(256) k_spans(const BatchDev *b) { spans_pass(b, false); }

// ------------------------------------------------------------------ shade --

__device__ __forceinline__ void bind_material(const SceneDev &s, uint32_t prim, Shader &sh)
{
    const uint4 *p = reinterpret_cast<const uint4 *>(s.pshade + prim); // PrimShade: one 32-byte load
    const uint4 a = p[0], c = p[1];
    sh.tex = reinterpret_cast<const uint32_t *>((unsigned long long)a.x | ((unsigned long long)a.y << 32));
    sh.tw = (int)a.z;
    sh.th = (int)a.w;
    sh.color = c.x;
    sh.shininess = (int)c.y;
}

// prepare_for_upper/lower_triangle, prepare_for_scanline and shade for the
// winner's progress values (renderer.cpp:433-493)
template <bool ALL_MODES = true>
__device__ __forceinline__ uint32_t shade_winner(Shader &sh, const LightsDev &L, const ViewDev &v, float4 rec)
{
    const uint32_t bits = __float_as_uint(rec.w);
    const bool llr = (bits & kBitLLR) != 0u;
    if (bits & kBitLower)
        sh_prepare_lower(sh, llr);
    else
        sh_prepare_upper(sh, llr);
    sh_prepare_scanline(sh, rec.y, rec.z);
    return sh_shade<ALL_MODES>(sh, L, v, rec.x);
}

// A winner of a near-clipped triangle: the clip vertices are rebuilt exactly
// as fill_triangle makes them; the progress values were recorded by the
// near-clip winner walk.  Rare, so kept out of line.
__device__ __noinline__ uint32_t shade_clip_rec(const ItemDev &it, uint32_t slot, float4 rec)
{
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
        if (it.v.shader == SGL_SHADER_FLAT_BILINEAR || it.v.shader == SGL_SHADER_FLAT_NEAREST ||
            it.v.shader == SGL_SHADER_FLAT)
            sh.flat_light = flat_light(sw, !ffv, *it.s.lights, it.v, sh.shininess);
        done = true;
    };
    clip_triangle(it, slot >> 1, emit);
    return done ? shade_winner(sh, *it.s.lights, it.v, rec) : 0u;
}

__device__ __forceinline__ uint32_t shade_clip_px(const ItemDev &it, uint32_t i, uint32_t slot)
{
    return shade_clip_rec(it, slot, it.prec[i]);
}

// The progress values of pixel (X, Y) (surface coordinates) from its winning
// triangle's set-up: the row's edges after their steps, the span and the
// qpixel chain up to X (renderer.cpp:474-493).  False when the span was wide
// enough to be binned (its winners were recorded by the span kernels).
__device__ __forceinline__ bool rec_replay(const TriRec *rp, const ViewDev &v, int inline_span, int X, int Y,
                                           float4 &out)
{
    const float4 *q = reinterpret_cast<const float4 *>(rp);
    const float4 q5 = q[5], q6 = q[6];
    const int y_s = __float_as_int(q5.y), y_l = __float_as_int(q5.z), n_u = __float_as_int(q5.w);
    const uint32_t flags = __float_as_uint(q6.y);
    const int k = (Y >= y_s && Y < y_s + n_u) ? Y - y_s : n_u + (Y - y_l);
    const float4 q0 = q[0], q1 = q[1], q4 = q[4];
    const float lg[6] = {q0.x, q0.y, q0.z, q0.w, q1.x, q1.y};
    float sh[6];
    if (k < n_u) {
        const float4 q2 = q[2];
        sh[0] = q1.z; sh[1] = q1.w; sh[2] = q2.x; sh[3] = q2.y; sh[4] = q2.z; sh[5] = q2.w;
    } else {
        const float4 q3 = q[3];
        sh[0] = q3.x; sh[1] = q3.y; sh[2] = q3.z; sh[3] = q3.w; sh[4] = q4.x; sh[5] = q4.y;
    }
    RowIn r;
    row_in(r, k, lg, sh, q4.z, q4.w, q5.x, y_s, y_l, n_u, flags);
    RowSpan sp;
    row_span(r, v.x, v.w, sp);
    if (sp.x2 - sp.x1 > inline_span)
        return false;
    Interp it;
    float pl, pr;
    span_interp(sp, it, pl, pr, X - sp.x1);
    out = make_float4(it.alpha, pl, pr, __uint_as_float(r.bits));
    return true;
}

template <bool ALL_MODES>
__device__ __forceinline__ uint32_t shade_rec(const ItemDev &it, uint4 q7, uint32_t flags, float4 rec);

// The colour of one winning fragment: pixel i of item `item`, won by `slot`.
template <bool ALL_MODES>
__device__ __forceinline__ uint32_t shade_winner_impl(const BatchDev *b, uint32_t item, uint32_t i, uint32_t slot,
                                                     bool overflow)
{
    const ItemDev &it = b->items[item];
    const ViewDev &v = it.v;
    const uint32_t r = __ldg(b->tri_base + item) + (slot >> 1);
    if (!in_bounds(r < b->list_cap, CHK_REC, r))
        return 0u;
    const TriRec *rp = b->recs + r;
    const uint4 q6 = reinterpret_cast<const uint4 *>(rp)[6];
    const uint4 q7 = reinterpret_cast<const uint4 *>(rp)[7];
    const uint32_t flags = q6.y;
    if (flags == kRecClip)
        return shade_clip_px(it, i, slot);
    const int y = (int)(i / (uint32_t)v.w), x = (int)(i - (uint32_t)y * (uint32_t)v.w);
    float4 rec;
    if (overflow || (flags & kRecTall) || !rec_replay(rp, v, b->inline_span, x + v.x, y + v.y, rec))
        rec = it.prec[i]; // recorded by the span kernels (or the overflow winner walk)
    return shade_rec<ALL_MODES>(it, q7, flags, rec);
}

// The colour of a fragment of a set-up triangle (vertices and primitive
// `q7`, TriRec flags `flags`) at the progress values `rec`.
template <bool ALL_MODES>
__device__ __forceinline__ uint32_t shade_rec(const ItemDev &it, uint4 q7, uint32_t flags, float4 rec)
{
    const ViewDev &v = it.v;
    Shader sh;
    bind_material(it.s, q7.w, sh);
    const float4 w0 = it.s.wpos[q7.x], w1 = it.s.wpos[q7.y], w2 = it.s.wpos[q7.z];
    const float4 n0 = it.s.wnrm[q7.x], n1 = it.s.wnrm[q7.y], n2 = it.s.wnrm[q7.z];
    const float2 u0 = it.s.uv[q7.x], u1 = it.s.uv[q7.y], u2 = it.s.uv[q7.z];
    const V3 sw[3] = {mk3(w0.x, w0.y, w0.z), mk3(w1.x, w1.y, w1.z), mk3(w2.x, w2.y, w2.z)};
    const V3 sn[3] = {mk3(n0.x, n0.y, n0.z), mk3(n1.x, n1.y, n1.z), mk3(n2.x, n2.y, n2.z)};
    const V2 su[3] = {mk2(u0.x, u0.y), mk2(u1.x, u1.y), mk2(u2.x, u2.y)};
    sh_prepare_triangle(sh, sw, sn, su, (flags & kRecFFV) == 0u);
    if (ALL_MODES &&
        (v.shader == SGL_SHADER_FLAT_BILINEAR || v.shader == SGL_SHADER_FLAT_NEAREST || v.shader == SGL_SHADER_FLAT))
        sh.flat_light = flat_light(sw, (flags & kRecFFV) == 0u, *it.s.lights, v, sh.shininess);
    return shade_winner<ALL_MODES>(sh, *it.s.lights, v, rec);
}



// Per pixel: the background of viewport_t::clear (viewport.cpp:88-113) or the
// colour of the winning fragment, and its depth.  A block takes TILE x TILE
// tiles; background pixels are written at once and winners are queued in
// shared memory, so that the shading runs on full warps.  The depth keys read
// are reset to empty for the next launch sequence (unless kept for debug).
constexpr int kShadeThreads = 256;
#ifndef SGL_SHADE_MIN_BLOCKS
#define SGL_SHADE_MIN_BLOCKS 5 // resident blocks per SM the shade is compiled for
#endif
template <int TILE, bool ALL_MODES>
__global__ void __launch_bounds__(kShadeThreads, SGL_SHADE_MIN_BLOCKS) k_shade(const BatchDev *b)
{
    __shared__ uint4 queue[2 * kShadeThreads];
    __shared__ int qn;
    const int lane = threadIdx.x & 31;
    if (threadIdx.x == 0)
        qn = 0;
    __syncthreads();
    __shared__ uint32_t tile_next;
    const bool overflow = *counter32(b, C_OVERFLOW) != 0u;
    const bool keep = b->keep_keys != 0;
    int item = -1;
    uint32_t lo = 0, hi = 0;
    // Tiles come from kQueues queues (queue q holds tiles q, q + kQueues,
    // ...; block b draws from queue b % kQueues); the next tile is fetched
    // while this one is shaded (the barriers of the loop order the exchange).
    const uint32_t qb = blockIdx.x % kQueues;
    uint32_t *tile_q = counter32(b, C_SHADE_Q + 32 * (int)qb);
    if (threadIdx.x == 0)
        tile_next = qb + kQueues * atomicAdd(tile_q, 1u);
    __syncthreads();
    for (;;) {
        const uint32_t tg = tile_next;
        if (tg >= b->total_tiles)
            break;
        __syncthreads(); // every thread has read tile_next
        if (threadIdx.x == 0)
            tile_next = qb + kQueues * atomicAdd(tile_q, 1u);
        if (tg < lo || tg >= hi) {
            item = find_item(b->tile_base, b->n_items, tg);
            lo = __ldg(b->tile_base + item);
            hi = __ldg(b->tile_base + item + 1);
        }
        const ItemDev &it = b->items[item];
        const uint32_t tl = tg - lo;
        const int tx = (int)(tl % (uint32_t)it.tiles_x), ty = (int)(tl / (uint32_t)it.tiles_x);
        for (int p0 = 0; p0 < TILE * TILE; p0 += kShadeThreads) {
            const int p = p0 + (int)threadIdx.x;
            const int x = tx * TILE + p % TILE, y = ty * TILE + p / TILE;
            bool win = false;
            uint32_t i = 0;
            unsigned long long k = kEmptyKey;
            if (p < TILE * TILE && x < it.v.w && y < it.v.h) {
                i = (uint32_t)y * (uint32_t)it.v.w + (uint32_t)x;
                k = it.key[i];
                if (k == kEmptyKey) {
                    it.pixels[(long long)y * it.pitch_px + x] = 0u;
                    if (it.zbuf)
                        it.zbuf[i] = __uint_as_float(kMaxZBits);
                } else {
                    win = true;
                    if (it.zbuf)
                        it.zbuf[i] = __uint_as_float((uint32_t)(k >> 32));
                    if (!keep)
                        it.key[i] = kEmptyKey;
                }
            }
            const unsigned m = __ballot_sync(0xFFFFFFFFu, win);
            int wb = 0;
            if (lane == 0 && m)
                wb = atomicAdd(&qn, __popc(m));
            wb = __shfl_sync(0xFFFFFFFFu, wb, 0);
            if (win)
                queue[wb + __popc(m & ((1u << lane) - 1u))] = make_uint4(i, (uint32_t)item, (uint32_t)k, 0u);
            __syncthreads();
            const int have = qn;
            if (have >= kShadeThreads) {
                const uint4 e = queue[threadIdx.x];
                const ItemDev &ie = b->items[e.y];
                const ViewDev &ve = ie.v;
                const uint32_t c = shade_winner_impl<ALL_MODES>(b, e.y, e.x, e.z, overflow);
                const int yy = (int)(e.x / (uint32_t)ve.w), xx = (int)(e.x - (uint32_t)yy * (uint32_t)ve.w);
                if (in_bounds(yy < ve.h, CHK_PIXEL, e.x))
                    ie.pixels[(long long)yy * ie.pitch_px + xx] = c;
                __syncthreads();
                if ((int)threadIdx.x < have - kShadeThreads)
                    queue[threadIdx.x] = queue[kShadeThreads + threadIdx.x];
                __syncthreads();
                if (threadIdx.x == 0)
                    qn = have - kShadeThreads;
            }
            __syncthreads();
        }
    }
    if ((int)threadIdx.x < qn) {
        const uint4 e = queue[threadIdx.x];
        const ItemDev &ie = b->items[e.y];
        const uint32_t c = shade_winner_impl<ALL_MODES>(b, e.y, e.x, e.z, overflow);
        const int yy = (int)(e.x / (uint32_t)ie.v.w), xx = (int)(e.x - (uint32_t)yy * (uint32_t)ie.v.w);
        if (in_bounds(yy < ie.v.h, CHK_PIXEL, e.x))
            ie.pixels[(long long)yy * ie.pitch_px + xx] = c;
    }
}

// The same per-pixel work for a batch of one large view (kSeqWinList), in
// two passes.  k_classify streams the batch's depth keys (one contiguous pool
// in batch pixel order, kClassifyPx keys per thread in flight): empty pixels
// get the background colour and depth at once; a winner gets its depth, its
// key is reset to empty (unless kept for debug), and it is appended to the
// winner list in pixel order, with one atomic per block pass.  k_shade_wins
// then shades one winner per thread, without tiles or barriers.
constexpr int kClassifyPx = 8; // pixels per thread and block pass

__global__ void __launch_bounds__(256) k_classify(const BatchDev *b)
{
    static_assert(kClassifyPx % 4 == 0, "the counts divide among the scan warp's lanes");
    __shared__ uint32_t at[kClassifyPx * 8]; // per (pass row j, warp): winners, then their first list index
    __shared__ uint32_t base;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const bool keep = b->keep_keys != 0;
    const uint32_t total = b->total_px;
    int item = -1;
    uint32_t lo = 0, hi = 0;
    for (uint32_t c0 = blockIdx.x * (256u * kClassifyPx); c0 < total; c0 += gridDim.x * (256u * kClassifyPx)) {
        unsigned long long k[kClassifyPx];
#pragma unroll
        for (int j = 0; j < kClassifyPx; j++) {
            const uint32_t g = c0 + j * 256u + threadIdx.x;
            k[j] = g < total ? b->key_pool[g] : kEmptyKey;
        }
        unsigned m[kClassifyPx];
#pragma unroll
        for (int j = 0; j < kClassifyPx; j++) {
            const uint32_t g = c0 + j * 256u + threadIdx.x;
            bool win = false;
            if (g < total) {
                if (g < lo || g >= hi) {
                    item = find_item(b->px_base, b->n_items, g);
                    lo = __ldg(b->px_base + item);
                    hi = __ldg(b->px_base + item + 1);
                }
                const ItemDev &it = b->items[item];
                const uint32_t i = g - lo, w = (uint32_t)it.v.w;
                const uint32_t y = i / w, x = i - y * w;
                if (k[j] == kEmptyKey) {
                    it.pixels[(long long)y * it.pitch_px + x] = 0u;
                    if (it.zbuf)
                        it.zbuf[i] = __uint_as_float(kMaxZBits);
                } else {
                    win = true;
                    if (it.zbuf)
                        it.zbuf[i] = __uint_as_float((uint32_t)(k[j] >> 32));
                    if (!keep)
                        b->key_pool[g] = kEmptyKey;
                }
            }
            m[j] = __ballot_sync(0xFFFFFFFFu, win);
            if (lane == 0)
                at[j * 8 + warp] = __popc(m[j]);
        }
        __syncthreads();
        if (warp == 0) {
            // exclusive prefix of the counts in (j, warp) order, which is pixel
            // order: each lane takes kPerLane consecutive counts
            constexpr int kPerLane = kClassifyPx * 8 / 32;
            uint32_t a[kPerLane], sum = 0;
#pragma unroll
            for (int q = 0; q < kPerLane; q++) {
                a[q] = at[kPerLane * lane + q];
                sum += a[q];
            }
            uint32_t incl = sum;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t t = __shfl_up_sync(0xFFFFFFFFu, incl, d);
                if (lane >= d)
                    incl += t;
            }
            uint32_t run = incl - sum;
#pragma unroll
            for (int q = 0; q < kPerLane; q++) {
                at[kPerLane * lane + q] = run;
                run += a[q];
            }
            if (lane == 31)
                base = incl ? atomicAdd(counter32(b, C_WINS), incl) : 0u;
        }
        __syncthreads();
        const unsigned below = (1u << lane) - 1u;
#pragma unroll
        for (int j = 0; j < kClassifyPx; j++)
            if (m[j] & (1u << lane)) {
                const uint32_t g = c0 + j * 256u + threadIdx.x;
                const uint32_t e = base + at[j * 8 + warp] + __popc(m[j] & below);
                if (in_bounds(e < total, CHK_PIXEL, e))
                    b->wins[e] = make_uint2(g, (uint32_t)k[j]);
            }
        __syncthreads(); // `at` and `base` are reused by the next pass
    }
}

template <bool ALL_MODES>
__global__ void __launch_bounds__(kShadeThreads, SGL_SHADE_MIN_BLOCKS) k_shade_wins(const BatchDev *b)
{
    const uint32_t n = *counter32(b, C_WINS);
    const bool overflow = *counter32(b, C_OVERFLOW) != 0u;
    int item = -1;
    uint32_t lo = 0, hi = 0;
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < n; e += gridDim.x * blockDim.x) {
        const uint2 wn = b->wins[e];
        if (wn.x < lo || wn.x >= hi) {
            item = find_item(b->px_base, b->n_items, wn.x);
            lo = __ldg(b->px_base + item);
            hi = __ldg(b->px_base + item + 1);
        }
        const ItemDev &it = b->items[item];
        const uint32_t i = wn.x - lo;
        const uint32_t c = shade_winner_impl<ALL_MODES>(b, (uint32_t)item, i, wn.y, overflow);
        const uint32_t y = i / (uint32_t)it.v.w, x = i - y * (uint32_t)it.v.w;
        if (in_bounds(y < (uint32_t)it.v.h, CHK_PIXEL, i))
            it.pixels[(long long)y * it.pitch_px + x] = c;
    }
}

// ------------------------------------------------------------ depth of field --

// The fragment pool was too small: nothing is written, the host renders again.
__device__ __forceinline__ bool frags_overflowed(const BatchDev *b)
{
    return *frag_counter(b) > (unsigned long long)b->frag_cap;
}

__constant__ float2 c_dof_taps[SGL_DOF_TAPS];

// Circle of confusion of pixel i of a depth-of-field item.
__device__ __forceinline__ float dof_radius(const ItemDev &it, uint32_t i)
{
    const float zp = it.zbuf[i];
    const float zv = (zp - it.p23) / it.p22;
    float r = (it.dof_ka * fabsf(zv - it.dof_focus)) / zv;
    if (!(r >= 0.0f && r <= it.dof_rmax))
        r = it.dof_rmax;
    return r;
}

__device__ __forceinline__ uint32_t dof_average(uint32_t centre, uint32_t sb, uint32_t sg, uint32_t sr)
{
    return (centre & 0xFF000000u) | (((sr + 16u) / 32u) << 16) | (((sg + 16u) / 32u) << 8) | ((sb + 16u) / 32u);
}

// Depth-of-field gather (replaces post_shader_depth_box,
// swegl/render/post_shaders.hpp:51-132).  Per pixel: view-space depth from the
// z-buffer, z = (z' - P23) / P22; circle of confusion r = K*A*|z - F| / z
// pixels, clamped to [0, max]; the mean of 32 taps of the golden-angle
// pattern (sgl_dof_taps.h) at offsets r * tap rounded to the nearest integer
// (ties to even: one conversion instruction), clamped to the
// viewport, with integer sums rounded half up.  Every step is exact integer
// or IEEE float arithmetic, so the CPU oracle gives the same bits.
//
// A block takes kDofTile x kDofTile tiles of the items that ask for the
// gather and stages the tile with its halo (the taps reach at most
// ceil(max_radius) pixels: every tap component is below 1), clamped to the
// view as the taps are, in shared memory (rows kDofPitch apart); the 32 taps
// of each pixel then read shared memory without further clamping.  Views whose reach exceeds
// kDofMaxHalo gather from the colour buffer.
constexpr int kDofBlocks = 5; // resident blocks per SM (shared memory: 37 KB each)

__global__ void __launch_bounds__(256, kDofBlocks) k_dof(const BatchDev *b)
{
    if (frags_overflowed(b))
        return; // a layered view whose fragment pool was too small: rendered again
    __shared__ uint32_t halo[kDofPitch * kDofPitch];
    __shared__ uint32_t claim[2]; // this tile and the next (tiles cost from a copy to a full gather)
    int item = -1;
    uint32_t lo = 0, hi = 0;
    if (threadIdx.x == 0)
        claim[0] = atomicAdd(counter32(b, C_DOF_NEXT), 1u);
    __syncthreads();
    for (int cb = 0;; cb ^= 1) {
        const uint32_t tg = claim[cb];
        if (tg >= b->total_dof_tiles)
            break;
        if (threadIdx.x == 0)
            claim[cb ^ 1] = atomicAdd(counter32(b, C_DOF_NEXT), 1u);
        if (tg < lo || tg >= hi) {
            item = find_item(b->dof_base, b->n_items, tg);
            lo = __ldg(b->dof_base + item);
            hi = __ldg(b->dof_base + item + 1);
        }
        const ItemDev &it = b->items[item];
        const int w = it.v.w, h = it.v.h;
        const uint32_t tl = tg - lo;
        const int x0 = (int)(tl % (uint32_t)it.dof_tiles_x) * kDofTile;
        const int y0 = (int)(tl / (uint32_t)it.dof_tiles_x) * kDofTile;
        const int R = it.dof_halo;
        const int S = kDofTile + 2 * R;
        if (R >= 0) {
            // rows of the halo to warps, columns to lanes (S <= 96: 3 per lane)
            const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
            int c0 = x0 - R + lane, c1 = c0 + 32, c2 = c0 + 64;
            c0 = c0 < 0 ? 0 : (c0 >= w ? w - 1 : c0);
            c1 = c1 < 0 ? 0 : (c1 >= w ? w - 1 : c1);
            c2 = c2 < 0 ? 0 : (c2 >= w ? w - 1 : c2);
            // the staged pixels' common value, if they all have one
            const uint32_t ref = __ldg(it.dof_src + (size_t)y0 * it.dof_src_pitch + x0);
            bool same = true;
#pragma unroll 4
            for (int yy = warp; yy < S; yy += 8) {
                int sy = y0 - R + yy;
                sy = sy < 0 ? 0 : (sy >= h ? h - 1 : sy);
                const uint32_t *row = it.dof_src + (size_t)sy * it.dof_src_pitch;
                uint32_t *dst = halo + yy * kDofPitch;
                if (lane < S) {
                    const uint32_t v = __ldg(row + c0);
                    dst[lane] = v;
                    same &= v == ref;
                }
                if (lane + 32 < S) {
                    const uint32_t v = __ldg(row + c1);
                    dst[lane + 32] = v;
                    same &= v == ref;
                }
                if (lane + 64 < S) {
                    const uint32_t v = __ldg(row + c2);
                    dst[lane + 64] = v;
                    same &= v == ref;
                }
            }
            if (__syncthreads_and(same)) {
                // Every tap of every pixel of the tile reads the value ref:
                // 32 equal channels c sum to 32 c, and (32 c + 16) / 32 = c,
                // alpha is the centre's: the gather leaves ref unchanged.
                for (int p = threadIdx.x; p < kDofTile * kDofTile; p += blockDim.x) {
                    const int x = x0 + (p & (kDofTile - 1)), y = y0 + p / kDofTile;
                    if (x < w && y < h)
                        it.dof_out[(size_t)y * it.dof_pitch + x] = ref;
                }
                __syncthreads(); // the halo is reused by the next tile, claim[cb ^ 1] is written
                continue;
            }
        }
        if (R >= 0) {
            // Warp w takes rows w, w + 8, w + 16 and w + 24 of the tile, a lane
            // one column.  The sums are exact integers, so the taps may be
            // taken in any order: rb sums bytes 0 and 2 in two 16-bit lanes
            // (32 x 255 fits), g sums whole pixels modulo 2^32, so that bits
            // 8..23 of g - rb are the sum of byte 1 (below 2^24 after the
            // shift: byte 3's sum lands at bit 24 and up); alpha is the
            // centre's.
            const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
            const int x = x0 + lane;
            const bool valid = x < w;
            const int xs = valid ? x : x0; // lanes past the view's right edge work on a pixel inside
            if (y0 + warp < h) {
                float r[4];
                bool uniform = true;
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int y = y0 + warp + 8 * j;
                    r[j] = y < h ? dof_radius(it, (uint32_t)y * (uint32_t)w + (uint32_t)xs) : 0.0f;
                }
                const float r0 = __shfl_sync(0xFFFFFFFFu, r[0], 0);
#pragma unroll
                for (int j = 0; j < 4; j++)
                    uniform &= !valid || y0 + warp + 8 * j >= h || r[j] == r0;
                // the halo holds the view-clamped pixels, so a tap needs no
                // clamp: |offset| <= ceil(r) <= R keeps it inside
                const uint32_t *c = halo + (warp + R) * kDofPitch + (xs - x0 + R);
                uint32_t rb[4] = {0u, 0u, 0u, 0u}, g[4] = {0u, 0u, 0u, 0u};
                if (__all_sync(0xFFFFFFFFu, uniform)) {
                    // one radius for the warp's 128 pixels (the clamped radius,
                    // or the empty background's): lane k makes tap k's offset
                    // once, and each offset serves the four rows
                    static_assert(SGL_DOF_TAPS == 32, "one tap per lane");
                    const float2 t = c_dof_taps[lane];
                    const int off = __float2int_rn(r0 * t.y) * kDofPitch + __float2int_rn(r0 * t.x);
#pragma unroll 4
                    for (int k = 0; k < SGL_DOF_TAPS; k++) {
                        const uint32_t *q = c + __shfl_sync(0xFFFFFFFFu, off, k);
#pragma unroll
                        for (int j = 0; j < 4; j++) {
                            const uint32_t v = q[8 * j * kDofPitch];
                            rb[j] += v & 0x00FF00FFu;
                            g[j] += v;
                        }
                    }
                } else {
#pragma unroll
                    for (int j = 0; j < 4; j++) {
                        if (y0 + warp + 8 * j >= h)
                            break; // the whole warp
                        const uint32_t *cj = c + 8 * j * kDofPitch;
                        const float rj0 = __shfl_sync(0xFFFFFFFFu, r[j], 0);
                        if (__all_sync(0xFFFFFFFFu, !valid || r[j] == rj0)) {
                            const float2 t = c_dof_taps[lane];
                            const int off = __float2int_rn(rj0 * t.y) * kDofPitch + __float2int_rn(rj0 * t.x);
#pragma unroll 8
                            for (int k = 0; k < SGL_DOF_TAPS; k++) {
                                const uint32_t v = cj[__shfl_sync(0xFFFFFFFFu, off, k)];
                                rb[j] += v & 0x00FF00FFu;
                                g[j] += v;
                            }
                        } else {
#pragma unroll 8
                            for (int k = 0; k < SGL_DOF_TAPS; k++) {
                                const float2 t = c_dof_taps[k];
                                const uint32_t v = cj[__float2int_rn(r[j] * t.y) * kDofPitch + __float2int_rn(r[j] * t.x)];
                                rb[j] += v & 0x00FF00FFu;
                                g[j] += v;
                            }
                        }
                    }
                }
#pragma unroll
                for (int j = 0; j < 4; j++) {
                    const int y = y0 + warp + 8 * j;
                    if (valid && y < h)
                        it.dof_out[(size_t)y * it.dof_pitch + x] =
                            dof_average(c[8 * j * kDofPitch], rb[j] & 0xFFFFu, ((g[j] - rb[j]) >> 8) & 0xFFFFu,
                                        rb[j] >> 16);
                }
            }
        } else {
            for (int p = threadIdx.x; p < kDofTile * kDofTile; p += blockDim.x) {
                const int x = x0 + (p & (kDofTile - 1)), y = y0 + p / kDofTile;
                if (y >= h)
                    continue; // the whole warp
                const bool valid = x < w;
                const int xs = valid ? x : x0;
                const float r = dof_radius(it, (uint32_t)y * (uint32_t)w + (uint32_t)xs);
                uint32_t sb = 0, sg = 0, sr = 0;
#pragma unroll 8
                for (int k = 0; k < SGL_DOF_TAPS; k++) {
                    const float2 t = c_dof_taps[k];
                    int sx = xs + __float2int_rn(r * t.x), sy = y + __float2int_rn(r * t.y);
                    sx = sx < 0 ? 0 : (sx >= w ? w - 1 : sx);
                    sy = sy < 0 ? 0 : (sy >= h ? h - 1 : sy);
                    const uint32_t v = __ldg(it.dof_src + (size_t)sy * it.dof_src_pitch + sx);
                    sb += v & 0xFFu;
                    sg += (v >> 8) & 0xFFu;
                    sr += (v >> 16) & 0xFFu;
                }
                if (valid)
                    it.dof_out[(size_t)y * it.dof_pitch + x] =
                        dof_average(it.dof_src[(size_t)y * it.dof_src_pitch + xs], sb, sg, sr);
            }
        }
        __syncthreads(); // the halo is reused by the next tile, claim[cb ^ 1] is written
    }
}

// The gather's input for a view with transparency layers: its rectangle of
// the surface after the layer passes (the flatten and copy write the surface
// at the reference's offsets, so the rectangle is read back whole), copied
// to the scratch buffer, since the gather writes the rectangle in place.
__global__ void __launch_bounds__(256) k_dof_source(const BatchDev *b)
{
    if (frags_overflowed(b))
        return;
    const ItemDev &it = b->items[0];
    const int w = it.v.w;
    const uint32_t total = (uint32_t)w * (uint32_t)it.v.h;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const int y = (int)(i / (uint32_t)w), x = (int)(i - (uint32_t)y * (uint32_t)w);
        it.dof_src[(size_t)y * it.dof_src_pitch + x] = it.dof_out[(long long)y * it.dof_pitch + x];
    }
}

// ------------------------------------------------------ transparency layers --
//
// A view with transparency layers (renderer.cpp:494-550) keeps per pixel the
// opaque depth and colour and up to `layers` transparent fragments sorted by
// depth, layer 0 the farthest.  The outcome depends on the draw order only
// through depth ties, so it can be computed from the pixel's fragments taken
// in any order:
//  - the screen gets the first drawn of the nearest opaque (alpha 255)
//    fragments, as without layers, and the depth buffer its depth;
//  - the layers hold the `layers` nearest transparent fragments strictly in
//    front of it, nearer meaning a smaller depth or, at equal depth, drawn
//    later (an insertion goes in front of the equal depths already there,
//    and when every layer is used the farthest is dropped).
// The capture walk chains every fragment of a pixel; the resolve takes a
// pixel's chain in (depth, draw order), shading fragments up to the first
// opaque one.  The flatten and copy passes follow viewport_t::flatten
// (viewport.cpp:43-86) and post_shader_t's copy of the first layer to the
// screen (post_shaders.hpp:22-47).  A layered batch holds one view.


// blend (src/render/colors.cpp:39-57): back * (256 - a) / 256 + front * a / 256
// truncated, which is exact in integers (both terms are multiples of 1/256).
__device__ __forceinline__ uint32_t blend_px(uint32_t back, uint32_t front)
{
    const uint32_t a = front >> 24, ba = back >> 24;
    const uint32_t na = 255u - ((255u - a) * (255u - ba) / 255u);
    if (a == 255u)
        return (front & 0x00FFFFFFu) | (na << 24);
    if (a == 0u)
        return (back & 0x00FFFFFFu) | (na << 24);
    uint32_t out = na << 24;
#pragma unroll
    for (int c = 0; c < 24; c += 8) {
        const uint32_t bc = (back >> c) & 0xFFu, fc = (front >> c) & 0xFFu;
        out |= ((bc * (256u - a) + fc * a) >> 8) << c;
    }
    return out;
}

// The fragments a triangle reserves (one per span pixel): the walk of its
// edges without the pixel loops.
struct FragCount {
    uint32_t slot; // unused (the walk's emit sets it)
    unsigned long long n;

    __device__ __forceinline__ bool active() const { return true; }
    __device__ __forceinline__ void drawn() {}
    __device__ __forceinline__ void span(int, int x1, int x2, const Side &, const Side &, uint32_t)
    {
        n += (unsigned long long)(x2 - x1);
    }
};

// Stores every fragment of its spans from the triangle's reserved range at
// `at` on (span_frags).  Spans longer than kFragInline are binned for
// k_frag_spans.
constexpr int kFragInline = 32;
struct FragVisitor {
    const BatchDev *b;
    const ItemDev *it;
    uint32_t slot;
    unsigned long long drawn_n, fragments;
    unsigned long long at;

    __device__ __forceinline__ bool active() const { return true; }
    __device__ __forceinline__ void drawn() { drawn_n++; }
    __device__ __forceinline__ void span(int y, int x1, int x2, const Side &Ls, const Side &Rs, uint32_t bits)
    {
        const unsigned long long n = (unsigned long long)(x2 - x1);
        fragments += n;
        const unsigned long long k = at;
        at += n;
        if (k + n > (unsigned long long)b->frag_cap)
            return; // counted, not stored: the pool is grown and the view rendered again
        if (n > (unsigned long long)kFragInline) {
            // a long span goes to the bins: its pixels are stored a warp at a time
            const uint32_t si = atomicAdd(counter32(b, C_SPANS), 1u);
            if (si < b->span_cap) {
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
                r.item = (uint32_t)k; // the span's first fragment (a layered batch has one item)
                b->spans[si] = r;
                return;
            }
        }
        const ViewDev &v = it->v;
        Interp q;
        q.init_self(Rs.x - Ls.x, Ls.it.value(), Rs.it.value());
        q.displace((float)x1 - Ls.x);
        span_frags(b, (uint32_t)((y - v.y) * v.w - v.x), slot, x1, x2, q, Ls.it.alpha, Rs.it.alpha, bits,
                   (uint32_t)k);
    }
};

// Fragment capture of the near-clipped triangles (the walk list is captured
// by k_walk<true, true>): one thread per triangle runs fill_triangle's clip cases
// and the fill_triangle_2 walk.  Each lane first counts its triangle's
// fragments; the warp then reserves its lanes' ranges with one atomic and
// walks again to store them.
__global__ void __launch_bounds__(256) k_frags(const BatchDev *b)
{
    const uint32_t c_raw = *counter32(b, C_CLIP);
    const uint32_t nc = c_raw < b->clip_cap ? c_raw : b->clip_cap;
    const int lane = threadIdx.x & 31;
    ItemAcc acc;
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i0 = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u; i0 < nc; i0 += stride) {
        const uint32_t i = i0 + (uint32_t)lane;
        const bool valid = i < nc;
        uint2 e = make_uint2(0u, 0u);
        if (valid)
            e = b->clip[b->clip_cap - 1 - i];
        const ItemDev &it = b->items[e.y];
        auto walk = [&](auto &vis) {
            if (!valid)
                return;
            auto emit = [&](uint32_t slot, const TV &a, const TV &c1, const TV &c2, bool) {
                vis.slot = slot;
                walk_sub(it.v, a.vp, c1.vp, c2.vp, vis);
            };
            clip_triangle(it, e.x, emit);
        };
        FragCount cnt{0u, 0ull};
        walk(cnt);
        unsigned long long incl = cnt.n;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long up = __shfl_up_sync(0xFFFFFFFFu, incl, o);
            if (lane >= o)
                incl += up;
        }
        unsigned long long base = 0;
        if (lane == 31 && incl)
            base = atomicAdd(frag_counter(b), incl);
        base = __shfl_sync(0xFFFFFFFFu, base, 31);
        FragVisitor vis{b, &it, 0u, 0ull, 0ull, base + incl - cnt.n};
        walk(vis);
        acc.add(b, e.y, vis.drawn_n, vis.fragments, valid);
    }
    acc.flush(b);
}

// The binned long spans of the capture, one warp each: the qpixel chain as in
// k_spans, then every lane stores its pixel's fragment.
__global__ void __launch_bounds__(256) k_frag_spans(const BatchDev *b)
{
    if (frags_overflowed(b))
        return;
    const uint32_t n_raw = *counter32(b, C_SPANS);
    const uint32_t n = n_raw < b->span_cap ? n_raw : b->span_cap;
    const ItemDev &it = b->items[0];
    const ViewDev &v = it.v;
    Frag *pool = b->frags;
    const int lane = threadIdx.x & 31;
    const uint32_t warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const uint32_t n_warps = (gridDim.x * blockDim.x) >> 5;
    for (uint32_t i = warp; i < n; i += n_warps) {
        const SpanRec r = b->spans[i];
        const int y = (int)(r.y_bits & kYMask);
        const uint32_t row_px = (uint32_t)((y - v.y) * v.w - v.x);
        const float fb = __uint_as_float(r.y_bits & ~kYMask);
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
            const bool keep = !below_near(z) && __float_as_uint(z) < kMaxZBits;
            const uint32_t at = r.item + (uint32_t)(x - r.x1);
            reinterpret_cast<float4 *>(pool + at)[0] = make_float4(alpha, r.progL, r.progR, fb);
            reinterpret_cast<uint4 *>(pool + at)[1] =
                make_uint4(__float_as_uint(z), r.slot, keep ? row_px + (uint32_t)x : kFragEnd, 0u);
        }
    }
}

// Chains the stored fragments to their pixels: one thread per pool entry
// swaps itself into its pixel's list head and keeps the previous head as its
// successor (the chain order is free: the resolve orders by depth and slot).
__global__ void __launch_bounds__(256) k_link(const BatchDev *b)
{
    if (frags_overflowed(b))
        return;
    const uint32_t n = (uint32_t)*frag_counter(b);
    uint32_t *head = b->items[0].frag_head;
    uint32_t *meta = reinterpret_cast<uint32_t *>(b->frags);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        uint32_t *next = meta + 8 * (size_t)i + 6; // Frag::next
        const uint32_t px = *next;
        if (px != kFragEnd)
            *next = atomicExch(head + px, i);
    }
}

// The colour of a captured fragment.
template <bool ALL_MODES>
__device__ __forceinline__ uint32_t shade_frag(const BatchDev *b, const ItemDev &it, uint32_t item, uint32_t slot,
                                               float4 rec)
{
    const uint4 *q = reinterpret_cast<const uint4 *>(b->recs + __ldg(b->tri_base + item) + (slot >> 1));
    const uint4 q6 = q[6];
    if (q6.y == kRecClip)
        return shade_clip_rec(it, slot, rec);
    return shade_rec<ALL_MODES>(it, q[7], q6.y, rec);
}

// One pixel with fragments: the opaque winner to the screen and the depth
// buffer, the transparent layers in front of it merged into the first one
// (viewport_t::flatten(front, back), viewport.cpp:43-51).
template <bool ALL_MODES>
__device__ __forceinline__ void resolve_pixel(const BatchDev *b, const ItemDev &it, uint32_t i)
{
    const int w = it.v.w, n_layers = it.layers;
    const Frag *pool = b->frags;
    const uint32_t head = it.frag_head[i];
    uint32_t lz[SGL_MAX_LAYERS], ls[SGL_MAX_LAYERS], lc[SGL_MAX_LAYERS]; // kept, nearest first
    int nt = 0;
    uint32_t wz = kMaxZBits, wc = 0u;
    unsigned long long prev = 0ull;
    bool first = true;
    // the first kChainRegs fragments of the chain are held in registers
    constexpr int kChainRegs = 4;
    unsigned long long ck[kChainRegs];
    uint32_t cf[kChainRegs];
    int held = 0;
    uint32_t rest = head; // the chain beyond the held fragments
#pragma unroll
    for (int k = 0; k < kChainRegs; k++) {
        if (rest != kFragEnd) {
            const uint4 m = reinterpret_cast<const uint4 *>(pool + rest)[1];
            ck[k] = ((unsigned long long)m.x << 32) | m.y;
            cf[k] = rest;
            held = k + 1;
            rest = m.z;
        }
    }
    for (;;) {
        // the next fragment in (depth, draw order)
        unsigned long long best = ~0ull;
        uint32_t bi = kFragEnd;
#pragma unroll
        for (int k = 0; k < kChainRegs; k++)
            if (k < held && (first || ck[k] > prev) && ck[k] < best) {
                best = ck[k];
                bi = cf[k];
            }
        for (uint32_t f = rest; f != kFragEnd;) {
            const uint4 m = reinterpret_cast<const uint4 *>(pool + f)[1];
            const unsigned long long key = ((unsigned long long)m.x << 32) | m.y;
            if ((first || key > prev) && key < best) {
                best = key;
                bi = f;
            }
            f = m.z;
        }
        if (bi == kFragEnd)
            break;
        first = false;
        prev = best;
        const uint32_t z = (uint32_t)(best >> 32), slot = (uint32_t)best;
        const uint32_t c = shade_frag<ALL_MODES>(b, it, 0u, slot, reinterpret_cast<const float4 *>(pool + bi)[0]);
        if ((c >> 24) == 255u) {
            wz = z;
            wc = c;
            while (nt > 0 && lz[nt - 1] == z)
                nt--; // not strictly in front
            break;
        }
        if (nt == n_layers && (z > lz[nt - 1] || (z == lz[nt - 1] && slot < ls[nt - 1])))
            continue; // farther than every kept layer
        int k = nt < n_layers ? nt : n_layers - 1;
        while (k > 0 && (lz[k - 1] > z || (lz[k - 1] == z && ls[k - 1] < slot))) {
            lz[k] = lz[k - 1];
            ls[k] = ls[k - 1];
            lc[k] = lc[k - 1];
            k--;
        }
        lz[k] = z;
        ls[k] = slot;
        lc[k] = c;
        if (nt < n_layers)
            nt++;
    }
    const int y = (int)(i / (uint32_t)w), x = (int)(i - (uint32_t)y * (uint32_t)w);
    it.pixels[(long long)y * it.pitch_px + x] = wc; // 0 = viewport_t::clear's background
    if (it.zbuf)
        it.zbuf[i] = __uint_as_float(wz);
    uint32_t l0 = nt > 0 ? lc[nt - 1] : 0u;
    for (int k = 1; k < nt; k++) {
        const uint32_t f = lc[nt - 1 - k];
        if (f >> 24)
            l0 = blend_px(l0, f);
    }
    it.layer0[i] = l0;
}

// Per pixel of the layered view: pixels without fragments get the background
// at once, the others are queued in shared memory and resolved by full warps.
template <bool ALL_MODES>
__global__ void __launch_bounds__(256, 4) k_layers(const BatchDev *b)
{
    if (frags_overflowed(b))
        return;
    __shared__ uint32_t queue[2 * 256];
    __shared__ int qn;
    const int lane = threadIdx.x & 31;
    if (threadIdx.x == 0)
        qn = 0;
    __syncthreads();
    const ItemDev &it = b->items[0];
    const int w = it.v.w;
    const uint32_t total = (uint32_t)w * (uint32_t)it.v.h;
    for (uint32_t c0 = blockIdx.x * 256u; c0 < total; c0 += gridDim.x * 256u) {
        const uint32_t i = c0 + threadIdx.x;
        bool busy = false;
        if (i < total) {
            if (it.frag_head[i] == kFragEnd) {
                const int y = (int)(i / (uint32_t)w), x = (int)(i - (uint32_t)y * (uint32_t)w);
                it.pixels[(long long)y * it.pitch_px + x] = 0u; // viewport_t::clear's background
                if (it.zbuf)
                    it.zbuf[i] = __uint_as_float(kMaxZBits);
                it.layer0[i] = 0u;
            } else {
                busy = true;
            }
        }
        const unsigned m = __ballot_sync(0xFFFFFFFFu, busy);
        int wb = 0;
        if (lane == 0 && m)
            wb = atomicAdd(&qn, __popc(m));
        wb = __shfl_sync(0xFFFFFFFFu, wb, 0);
        if (busy)
            queue[wb + __popc(m & ((1u << lane) - 1u))] = i;
        __syncthreads();
        const int have = qn;
        if (have >= 256) {
            resolve_pixel<ALL_MODES>(b, it, queue[threadIdx.x]);
            __syncthreads();
            if ((int)threadIdx.x < have - 256)
                queue[threadIdx.x] = queue[256 + threadIdx.x];
            __syncthreads();
            if (threadIdx.x == 0)
                qn = have - 256;
        }
        __syncthreads();
    }
    if ((int)threadIdx.x < qn)
        resolve_pixel<ALL_MODES>(b, it, queue[threadIdx.x]);
}

// viewport_t::flatten(front) (viewport.cpp:53-79): view pixel (x, y) reads
// the surface at row y, column x.
__global__ void __launch_bounds__(256) k_flatten(const BatchDev *b)
{
    if (frags_overflowed(b))
        return;
    const ItemDev &it = b->items[0];
    const int w = it.v.w;
    const uint32_t total = (uint32_t)w * (uint32_t)it.v.h;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const int y = (int)(i / (uint32_t)w), x = (int)(i - (uint32_t)y * (uint32_t)w);
        const uint32_t back = it.surface[(long long)y * it.pitch_px + x];
        const uint32_t f = it.layer0[i];
        it.layer0[i] = (f >> 24) ? blend_px(back, f) : back;
    }
}

// post_shader_t::copy_first_transparency_layer_to_screen
// (post_shaders.hpp:22-31): view pixel (x, y) to surface row y + view y,
// column x.
__global__ void __launch_bounds__(256) k_copy_layer(const BatchDev *b)
{
    if (frags_overflowed(b))
        return;
    const ItemDev &it = b->items[0];
    const int w = it.v.w;
    const uint32_t total = (uint32_t)w * (uint32_t)it.v.h;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
        const int y = (int)(i / (uint32_t)w), x = (int)(i - (uint32_t)y * (uint32_t)w);
        it.surface[(long long)(y + it.v.y) * it.pitch_px + x] = it.layer0[i];
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
    if (s.pbox && s.n_prims)
        k_box<<<(s.n_prims + 7) / 8, 256, 0, st>>>(s, s.wpos, s.pbox);
    return cudaGetLastError();
}

cudaError_t launch_pose(const SceneDev &s, const float *node_world, const float *node_rs, float4 *wpos, float4 *wnrm,
                        float4 *pbox, cudaStream_t st)
{
    if (s.n_vertices == 0)
        return cudaSuccess;
    k_pose<<<grid_for(s.n_vertices, 256), 256, 0, st>>>(s, node_world, node_rs, wpos, wnrm);
    if (pbox && s.n_prims)
        k_box<<<(s.n_prims + 7) / 8, 256, 0, st>>>(s, wpos, pbox);
    return cudaGetLastError();
}

const char *prof_kernel_name(int k)
{
    static const char *names[kProfKernels] = {"k_geom",    "k_vertex",  "k_flags",  "k_compact", "k_setup",
                                              "k_walk",    "k_spans",   "k_winners", "k_shade",  "k_dof",
                                              "k_frags",   "k_layers",  "k_flatten", "k_copy_layer"};
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
            if (!(p->ran & (1u << k)))
                continue; // a stage this sequence skipped
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
    cudaError_t e = cudaMemcpyToSymbol(c_dof_taps, taps, sizeof taps);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_geom, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kGeomSmem);
    return e;
}

cudaError_t check_status(unsigned *code, unsigned long long *index, unsigned *count, bool reset, bool *compiled)
{
#ifdef SGL_BOUNDS_CHECK
    *compiled = true;
    unsigned long long first = 0;
    unsigned n = 0;
    cudaError_t e = cudaMemcpyFromSymbol(&first, g_check_first, sizeof first);
    if (e == cudaSuccess)
        e = cudaMemcpyFromSymbol(&n, g_check_count, sizeof n);
    if (e == cudaSuccess && reset) {
        const unsigned long long z0 = 0;
        const unsigned z1 = 0;
        e = cudaMemcpyToSymbol(g_check_first, &z0, sizeof z0);
        if (e == cudaSuccess)
            e = cudaMemcpyToSymbol(g_check_count, &z1, sizeof z1);
    }
    *code = (unsigned)(first >> 48);
    *index = first & 0xFFFFFFFFFFFFull;
    *count = n;
    return e;
#else
    *compiled = false;
    *code = 0;
    *index = 0;
    *count = 0;
    (void)reset;
    return cudaSuccess;
#endif
}

cudaError_t launch_dof(const BatchDev *b, cudaStream_t st)
{
    k_dof<<<sm_count() * kDofBlocks, 256, 0, st>>>(b);
    return cudaGetLastError();
}

cudaError_t launch_batch(const BatchDev *b, int tile, int flags, cudaStream_t st, int *launches, Profiler *prof)
{
    const bool timed = prof && prof->enabled;
    if (timed) {
        prof_collect(prof);
        for (int k = 0; k <= kProfKernels; k++)
            if (!prof->ev[k] && cudaEventCreate(&prof->ev[k]) != cudaSuccess)
                return cudaGetLastError();
    }
    if (timed)
        prof->ran = 0;
    auto mark = [&](int k) {
        if (timed)
            cudaEventRecord(prof->ev[k], st);
    };
    auto ran = [&](int k) {
        if (timed)
            prof->ran |= 1u << k;
    };
    const int sms = sm_count();
    int n = 0;
    mark(PK_GEOM);
    if (flags & kSeqFused) {
        k_geom<<<sms * kGeomBlocks * 2, kGeomWarps * 32, kGeomSmem, st>>>(b);
        ran(PK_GEOM);
        n++;
    }
    mark(PK_VERTEX);
    if (flags & kSeqSplit) {
        k_vertex<<<sms * 8, 256, 0, st>>>(b);
        ran(PK_VERTEX);
        mark(PK_FLAGS);
        k_flags<<<sms * 8, 256, 0, st>>>(b);
        ran(PK_FLAGS);
        mark(PK_COMPACT);
        k_compact<<<sms * 4, kCompactBlock, 0, st>>>(b);
        ran(PK_COMPACT);
        n += 3;
    } else {
        mark(PK_FLAGS);
        mark(PK_COMPACT);
    }
    mark(PK_SETUP);
    k_setup<<<sms * 8, 256, 0, st>>>(b);
    ran(PK_SETUP);
    n++;
    if (flags & kSeqLayers) {
        for (int k = PK_WALK; k <= PK_DOF; k++)
            mark(k);
        mark(PK_FRAGS);
        k_walk<true, true><<<sms * SGL_WALK_MIN_BLOCKS, kWalkWarps * 32, 0, st>>>(b); // (one view)
        k_frags<<<sms * 2, 256, 0, st>>>(b);
        k_frag_spans<<<sms * 4, 256, 0, st>>>(b);
        k_link<<<sms * 8, 256, 0, st>>>(b);
        ran(PK_FRAGS);
        mark(PK_LAYERS);
        if (flags & kSeqShaders)
            k_layers<true><<<sms * 4, 256, 0, st>>>(b);
        else
            k_layers<false><<<sms * 4, 256, 0, st>>>(b);
        ran(PK_LAYERS);
        mark(PK_FLATTEN);
        k_flatten<<<sms * 8, 256, 0, st>>>(b);
        ran(PK_FLATTEN);
        mark(PK_COPY);
        k_copy_layer<<<sms * 8, 256, 0, st>>>(b);
        ran(PK_COPY);
        n += 7;
        if (flags & kSeqDof) { // the gather over the view's rectangle, from a copy of it (timed with the copy)
            k_dof_source<<<sms * 8, 256, 0, st>>>(b);
            k_dof<<<sms * kDofBlocks, 256, 0, st>>>(b);
            n += 2;
        }
        if (timed) {
            cudaEventRecord(prof->ev[kProfKernels], st);
            prof->pending = true;
        }
        if (launches)
            *launches += n;
        return cudaGetLastError();
    }
    mark(PK_WALK);
    if (flags & kSeqOne)
        k_walk<false, true><<<sms * SGL_WALK_MIN_BLOCKS, kWalkWarps * 32, 0, st>>>(b);
    else
        k_walk<false, false><<<sms * SGL_WALK_MIN_BLOCKS, kWalkWarps * 32, 0, st>>>(b);
    ran(PK_WALK);
    n++;
    mark(PK_SPANS);
    k_spans<<<sms * 4, 256, 0, st>>>(b);
    ran(PK_SPANS);
    n++;
    mark(PK_WINNER);
    k_winners<<<sms * 4, 256, 0, st>>>(b);
    ran(PK_WINNER);
    n++;
    mark(PK_SHADE);
    // the kernel with every pixel shader only when a view asks for another
    // than the default, which then keeps all the registers
    const unsigned sg = sms * SGL_SHADE_MIN_BLOCKS;
    if (flags & kSeqWinList) {
        k_classify<<<sms * 8, 256, 0, st>>>(b);
        if (flags & kSeqShaders)
            k_shade_wins<true><<<sg, kShadeThreads, 0, st>>>(b);
        else
            k_shade_wins<false><<<sg, kShadeThreads, 0, st>>>(b);
        n++;
    } else if (flags & kSeqShaders) {
        if (tile == 8)
            k_shade<8, true><<<sg, kShadeThreads, 0, st>>>(b);
        else if (tile == 32)
            k_shade<32, true><<<sg, kShadeThreads, 0, st>>>(b);
        else
            k_shade<16, true><<<sg, kShadeThreads, 0, st>>>(b);
    } else {
        if (tile == 8)
            k_shade<8, false><<<sg, kShadeThreads, 0, st>>>(b);
        else if (tile == 32)
            k_shade<32, false><<<sg, kShadeThreads, 0, st>>>(b);
        else
            k_shade<16, false><<<sg, kShadeThreads, 0, st>>>(b);
    }
    ran(PK_SHADE);
    n++;
    mark(PK_DOF);
    if (flags & kSeqDof) {
        k_dof<<<sms * kDofBlocks, 256, 0, st>>>(b);
        ran(PK_DOF);
        n++;
    }
    for (int k = PK_FRAGS; k <= PK_COPY; k++)
        mark(k);
    if (timed) {
        cudaEventRecord(prof->ev[kProfKernels], st);
        prof->pending = true;
    }
    if (launches)
        *launches += n;
    return cudaGetLastError();
}

} // namespace sgl
