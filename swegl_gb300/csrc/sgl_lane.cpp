// sgl_lane.cpp — batches of views on one stream: descriptor staging, scratch
// pools, the launch sequence and its CUDA graphs.
#include <algorithm>
#include <cstring>
#include <vector>

#include <cuda_runtime.h>

#include "sgl.h"
#include "sgl_internal.h"
#include "sgl_runtime.h"

namespace sgl {

HostBuf::~HostBuf()
{
    if (ptr)
        cudaFreeHost(ptr);
}

cudaError_t HostBuf::ensure(size_t need)
{
    if (need <= bytes && ptr)
        return cudaSuccess;
    if (ptr)
        cudaFreeHost(ptr);
    ptr = nullptr;
    bytes = 0;
    size_t n = std::max<size_t>(need, 256);
    cudaError_t e = cudaHostAlloc(&ptr, n, cudaHostAllocDefault);
    if (e != cudaSuccess) {
        ptr = nullptr;
        return e;
    }
    bytes = n;
    return cudaSuccess;
}

static size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

size_t view_scratch_bytes(uint32_t n_vertices, uint32_t n_triangles, int w, int h)
{
    const size_t px = (size_t)w * h;
    return align_up(16 * (size_t)n_vertices, 256) + align_up(n_vertices, 256) + 8 * px + 16 * px  // ndc yes key prec
           + (px >= kWinListMinPixels ? 8 * px : 0)                                               // winner list
           + (8 + sizeof(TriRec) + 8) * (size_t)n_triangles + sizeof(SpanRec) * (px / 8 + 64)      // lists, set-ups, bins
           + 8 * px;                                                                               // dof colour, depth
}

Lane::~Lane()
{
    for (auto &sl : slots) {
        for (auto &gt : sl.graph)
            for (auto &g : gt)
                if (g)
                    cudaGraphExecDestroy(g);
        if (sl.staged)
            cudaEventDestroy(sl.staged);
        if (sl.done)
            cudaEventDestroy(sl.done);
    }
    if (own_stream && stream)
        cudaStreamDestroy(stream);
    if (capture_stream)
        cudaStreamDestroy(capture_stream);
}

sgl_status Lane::init(Ctx *ctx, int max_items_, cudaStream_t external, bool blocking)
{
    max_items = max_items_;
    CUDA_TRY(init_device_constants());
    if (external) {
        stream = external;
        own_stream = false;
    } else {
        CUDA_TRY(cudaStreamCreateWithFlags(&stream, blocking ? cudaStreamDefault : cudaStreamNonBlocking));
        own_stream = true;
    }
    for (auto &sl : slots) {
        CUDA_TRY(sl.d_items.ensure(sizeof(ItemDev) * (size_t)max_items));
        CUDA_TRY(sl.d_bases.ensure(sizeof(uint32_t) * kBaseArrays * ((size_t)max_items + 1)));
        CUDA_TRY(sl.d_batch.ensure(sizeof(BatchDev)));
        CUDA_TRY(sl.d_counters.ensure(sizeof(unsigned long long) * kCounterWords));
        CUDA_TRY(sl.d_item_counters.ensure(2 * sizeof(unsigned long long) * (size_t)max_items));
        CUDA_TRY(sl.h_items.ensure(sizeof(ItemDev) * (size_t)max_items));
        CUDA_TRY(sl.h_bases.ensure(sizeof(uint32_t) * kBaseArrays * ((size_t)max_items + 1)));
        CUDA_TRY(sl.h_batch.ensure(sizeof(BatchDev)));
        CUDA_TRY(sl.h_counters.ensure(sizeof(unsigned long long) * (kCounterWords + 2 * (size_t)max_items)));
        CUDA_TRY(cudaEventCreateWithFlags(&sl.staged, cudaEventDisableTiming));
        CUDA_TRY(cudaEventCreateWithFlags(&sl.done, cudaEventDisableTiming));
    }
    return SGL_OK;
}

sgl_status Lane::prepare(Ctx *ctx, const BatchEntry *e, int n, int tile, int inline_span, uint8_t *slot_flags,
                         int *slot_out)
{
    if (n <= 0 || n > max_items) {
        ctx->fail("batch of %d views; this lane takes 1..%d", n, max_items);
        return SGL_ERR_INVALID;
    }
    const int si = next;
    next = (next + 1) % kSlots;
    Slot &sl = slots[si];
    if (sl.used)
        CUDA_TRY(cudaEventSynchronize(sl.done)); // its staging buffers are free again
    // prefixes and pool offsets
    uint32_t *hb = (uint32_t *)sl.h_bases.ptr;
    uint32_t *vb = hb, *tb = hb + (n + 1), *pb = hb + 2 * (n + 1), *gb = hb + 3 * (n + 1), *fb = hb + 4 * (n + 1);
    uint32_t *gvb = hb + 5 * (n + 1), *gtb = hb + 6 * (n + 1);
    uint32_t *gcb = hb + 7 * (n + 1), *gib = hb + 8 * (n + 1), *gi = hb + 9 * (n + 1);
    uint64_t tv = 0, tt = 0, tp = 0, tg = 0, tf = 0, dof_px = 0, dofz_px = 0, tgv = 0, tgt = 0;
    // items of fused scenes, grouped by the vertex data they read (the scene's
    // world positions, or a posed request's own), groups in order of first use
    std::vector<const void *> grp_key;
    std::vector<std::vector<uint32_t>> grp_members;
    int geom_flags = 0;
    size_t ndc_off = 0, yes_off = 0;
    std::vector<size_t> ndc_at(n), yes_at(n), dof_at(n), dofz_at(n);
    for (int i = 0; i < n; i++) {
        const Scene &s = *e[i].scene;
        const sgl_view &v = e[i].view;
        vb[i] = (uint32_t)tv;
        tb[i] = (uint32_t)tt;
        pb[i] = (uint32_t)tp;
        gb[i] = (uint32_t)tg;
        fb[i] = (uint32_t)tf;
        gvb[i] = (uint32_t)tgv;
        gtb[i] = (uint32_t)tgt;
        if (s.dev.fused) {
            const void *key = e[i].wpos ? (const void *)e[i].wpos : (const void *)s.dev.wpos;
            size_t gk = 0;
            while (gk < grp_key.size() && grp_key[gk] != key)
                gk++;
            if (gk == grp_key.size()) {
                grp_key.push_back(key);
                grp_members.emplace_back();
            }
            grp_members[gk].push_back((uint32_t)i);
            geom_flags |= kSeqFused;
        }
        if (!s.dev.fused || s.dev.mixed) { // the general passes (of a mixed scene: its larger primitives)
            tgv += s.n_vertices;
            tgt += s.n_triangles;
            geom_flags |= kSeqSplit;
        }
        tv += s.n_vertices;
        tt += s.n_triangles;
        tp += (uint64_t)v.w * v.h;
        tg += (uint64_t)((v.w + tile - 1) / tile) * (uint64_t)((v.h + tile - 1) / tile);
        if (v.dof.enabled)
            tf += (uint64_t)((v.w + kDofTile - 1) / kDofTile) * (uint64_t)((v.h + kDofTile - 1) / kDofTile);
        ndc_at[i] = ndc_off;
        yes_at[i] = yes_off;
        ndc_off += align_up(s.n_vertices, 16);
        yes_off += align_up(s.n_vertices, 256);
        dof_at[i] = dof_px;
        dofz_at[i] = dofz_px;
        if (v.dof.enabled) {
            dof_px += align_up((size_t)v.w * v.h, 64);
            if (!e[i].zbuf)
                dofz_px += align_up((size_t)v.w * v.h, 64);
        }
    }
    // the fused pass's groups: chunks of kGeomWarps primitives, items
    uint64_t tc = 0;
    uint32_t n_grouped = 0;
    const int n_groups = (int)grp_key.size();
    for (int k = 0; k < n_groups; k++) {
        gcb[k] = (uint32_t)tc;
        gib[k] = n_grouped;
        const Scene &s = *e[grp_members[k][0]].scene;
        tc += (s.dev.n_prims + kGeomWarps - 1) / kGeomWarps;
        for (uint32_t it : grp_members[k])
            gi[n_grouped++] = it;
    }
    gcb[n_groups] = (uint32_t)tc;
    gib[n_groups] = n_grouped;
    if (tv >= (1ull << 32) || tt >= (1ull << 31) || tp >= (1ull << 32) || tg >= (1ull << 32) || tf >= (1ull << 32) ||
        tc >= (1ull << 31)) {
        ctx->fail("batch too large (%llu vertices, %llu triangles, %llu pixels)", (unsigned long long)tv,
                  (unsigned long long)tt, (unsigned long long)tp);
        return SGL_ERR_UNSUPPORTED;
    }
    vb[n] = (uint32_t)tv;
    tb[n] = (uint32_t)tt;
    pb[n] = (uint32_t)tp;
    gb[n] = (uint32_t)tg;
    fb[n] = (uint32_t)tf;
    gvb[n] = (uint32_t)tgv;
    gtb[n] = (uint32_t)tgt;
    const size_t span_cap = std::max<size_t>(65536, tp / 8);
    CUDA_TRY(ndc.ensure(sizeof(float4) * std::max<size_t>(ndc_off, 1)));
    CUDA_TRY(yes.ensure(std::max<size_t>(yes_off, 1)));
    const void *key_was = key.ptr;
    CUDA_TRY(key.ensure(sizeof(unsigned long long) * std::max<uint64_t>(tp, 1)));
    if (key.ptr != key_was || keys_dirty) {
        // a new pool, or one a debug render or a failed launch left dirty
        CUDA_TRY(cudaMemsetAsync(key.ptr, 0xFF, key.bytes, stream)); // kEmptyKey is all ones
        keys_dirty = false;
    }
    CUDA_TRY(prec.ensure(sizeof(float4) * std::max<uint64_t>(tp, 1)));
    // one large view: the shade goes through a winner list
    const bool win_list = n == 1 && tp >= kWinListMinPixels && e[0].view.layers == 0;
    if (win_list)
        CUDA_TRY(wins.ensure(sizeof(uint2) * tp));
    CUDA_TRY(list.ensure(sizeof(uint2) * std::max<uint64_t>(tt, 1)));
    CUDA_TRY(recs.ensure(sizeof(TriRec) * std::max<uint64_t>(tt, 1)));
    CUDA_TRY(tall.ensure(sizeof(uint32_t) * std::max<uint64_t>(tt, 1)));
    CUDA_TRY(spans.ensure(sizeof(SpanRec) * span_cap));
    if (dof_px) {
        CUDA_TRY(doftmp.ensure(4 * dof_px));
        if (dofz_px)
            CUDA_TRY(dofz.ensure(4 * dofz_px));
    }
    int seq_flags = geom_flags | (win_list ? kSeqWinList : 0) | (n == 1 ? kSeqOne : 0);
    int layers = 0;
    for (int i = 0; i < n; i++)
        layers = std::max(layers, e[i].view.layers);
    size_t frag_cap = 0;
    if (layers > 0) {
        // one view per layered batch: its flatten and copy passes read and
        // write the whole surface, in view order
        if (n != 1 || !e[0].surface) {
            ctx->fail("transparency layers take one view per launch sequence");
            return SGL_ERR_UNSUPPORTED;
        }
        frag_want = std::max<size_t>(frag_want, std::max<size_t>(4 * tp, 65536));
        CUDA_TRY(frags.ensure(sizeof(Frag) * frag_want));
        CUDA_TRY(frag_head.ensure(4 * tp));
        CUDA_TRY(layer0.ensure(4 * tp));
        CUDA_TRY(cudaMemsetAsync(frag_head.ptr, 0xFF, 4 * tp, stream)); // kFragEnd
        frag_cap = std::min<size_t>(frags.bytes / sizeof(Frag), 0xFFFFFFFFu);
        seq_flags |= kSeqLayers;
    }
    ItemDev *hi = (ItemDev *)sl.h_items.ptr;
    for (int i = 0; i < n; i++) {
        const BatchEntry &en = e[i];
        ItemDev it{};
        it.s = en.scene->dev;
        if (en.wpos) { // a posed request: its own world positions, normals and node matrices
            it.s.wpos = en.wpos;
            it.s.wnrm = en.wnrm;
            it.s.pbox = en.pbox;
            it.s.node_world = en.node_world;
            it.s.node_rs = en.node_rs;
        }
        it.v = make_view(en.view);
        it.ndc = (float4 *)ndc.ptr + ndc_at[i];
        it.yes = (uint8_t *)yes.ptr + yes_at[i];
        it.key = (unsigned long long *)key.ptr + pb[i];
        it.prec = (float4 *)prec.ptr + pb[i];
        it.pixels = en.rect_pixels;
        it.pitch_px = en.pitch_px;
        it.zbuf = en.zbuf;
        it.tiles_x = (en.view.w + tile - 1) / tile;
        it.tile_base = gb[i];
        if (en.view.dof.enabled) {
            // the shade kernel fills a scratch colour buffer; the gather writes
            // the target (a layered view: the layer passes write the surface,
            // then its rectangle is copied to the scratch buffer and gathered
            // back in place)
            const sgl_dof_desc &d = en.view.dof;
            seq_flags |= kSeqDof;
            it.dof = 1;
            it.dof_out = en.rect_pixels;
            it.dof_pitch = en.pitch_px;
            it.dof_src = (uint32_t *)doftmp.ptr + dof_at[i];
            it.dof_src_pitch = en.view.w;
            if (en.view.layers == 0) {
                it.pixels = it.dof_src;
                it.pitch_px = en.view.w;
            }
            if (!en.zbuf)
                it.zbuf = (float *)dofz.ptr + dofz_at[i];
            const float k = d.px_scale > 0.0f ? d.px_scale : (en.view.proj[5] * (float)en.view.h) / 2.0f;
            it.dof_focus = d.focus;
            it.dof_ka = k * d.aperture;
            it.dof_rmax = d.max_radius;
            it.p22 = en.view.proj[10];
            it.p23 = en.view.proj[11];
            it.dof_halo = dof_halo_of(d.max_radius);
            it.dof_tiles_x = (en.view.w + kDofTile - 1) / kDofTile;
        }
        if (en.view.shader != SGL_SHADER_PHONG_BILINEAR)
            seq_flags |= kSeqShaders;
        if (layers > 0) {
            it.layers = en.view.layers;
            it.surface = en.surface;
            it.frag_head = (uint32_t *)frag_head.ptr;
            it.layer0 = (uint32_t *)layer0.ptr;
        }
        hi[i] = it;
    }
    BatchDev *hbd = (BatchDev *)sl.h_batch.ptr;
    BatchDev bd{};
    bd.items = (const ItemDev *)sl.d_items.ptr;
    const uint32_t *db = (const uint32_t *)sl.d_bases.ptr;
    bd.tri_base = db + (n + 1); // (db[0 .. n]: the vertex prefix, read by nothing on the device)
    bd.px_base = db + 2 * (n + 1);
    bd.tile_base = db + 3 * (n + 1);
    bd.dof_base = db + 4 * (n + 1);
    bd.g_vtx_base = db + 5 * (n + 1);
    bd.g_tri_base = db + 6 * (n + 1);
    bd.grp_chunk_base = db + 7 * (n + 1);
    bd.grp_item_base = db + 8 * (n + 1);
    bd.grp_items = db + 9 * (n + 1);
    bd.n_groups = n_groups;
    bd.total_gvtx = (uint32_t)tgv;
    bd.total_gtri = (uint32_t)tgt;
    bd.total_chunks = (uint32_t)tc;
    bd.n_items = n;
    bd.inline_span = inline_span;
    bd.total_px = (uint32_t)tp;
    bd.total_tiles = (uint32_t)tg;
    bd.total_dof_tiles = (uint32_t)tf;
    bd.list = (uint2 *)list.ptr;
    bd.list_cap = (uint32_t)std::max<uint64_t>(tt, 1);
    bd.clip = (uint2 *)list.ptr; // shares the list buffer, filled from its end
    bd.clip_cap = bd.list_cap;
    bd.recs = (TriRec *)recs.ptr;
    bd.tall = (uint32_t *)tall.ptr;
    bd.keep_keys = slot_flags != nullptr; // debug renders read the keys back
    bd.key_pool = (unsigned long long *)key.ptr;
    bd.wins = win_list ? (uint2 *)wins.ptr : nullptr;
    sl.keep_keys = bd.keep_keys != 0;
    bd.spans = (SpanRec *)spans.ptr;
    bd.span_cap = (uint32_t)std::min<size_t>(spans.bytes / sizeof(SpanRec), 0xFFFFFFFFu);
    bd.counters = (unsigned long long *)sl.d_counters.ptr;
    bd.item_counters = (unsigned long long *)sl.d_item_counters.ptr;
    bd.slot_flags = slot_flags;
    bd.frags = (Frag *)frags.ptr;
    bd.frag_cap = (uint32_t)frag_cap;
    *hbd = bd;
    CUDA_TRY(cudaMemcpyAsync(sl.d_items.ptr, hi, sizeof(ItemDev) * n, cudaMemcpyHostToDevice, stream));
    CUDA_TRY(cudaMemcpyAsync(sl.d_bases.ptr, hb, sizeof(uint32_t) * kBaseArrays * (n + 1), cudaMemcpyHostToDevice, stream));
    CUDA_TRY(cudaMemcpyAsync(sl.d_batch.ptr, hbd, sizeof(BatchDev), cudaMemcpyHostToDevice, stream));
    CUDA_TRY(cudaMemsetAsync(sl.d_counters.ptr, 0, sizeof(unsigned long long) * kCounterWords, stream));
    CUDA_TRY(cudaMemsetAsync(sl.d_item_counters.ptr, 0, 2 * sizeof(unsigned long long) * n, stream));
    CUDA_TRY(cudaEventRecord(sl.staged, stream));
    sl.used = true;
    sl.n_items = n;
    sl.seq_flags = seq_flags;
    *slot_out = si;
    return SGL_OK;
}

static int tile_index(int tile) { return tile == 8 ? 0 : (tile == 32 ? 2 : 1); }

sgl_status Lane::launch(Ctx *ctx, int si, int tile, bool use_graph, int *launches, Profiler *prof)
{
    Slot &sl = slots[si];
    const BatchDev *db = (const BatchDev *)sl.d_batch.ptr;
    keys_dirty = true; // until the sequence is enqueued: its shade kernel empties the keys
    if (use_graph) {
        cudaGraphExec_t &g = sl.graph[tile_index(tile)][sl.seq_flags];
        if (!g) {
            // captured on a private stream (the caller's may be the legacy
            // default stream, which cannot be captured), launched on the caller's
            if (!capture_stream)
                CUDA_TRY(cudaStreamCreateWithFlags(&capture_stream, cudaStreamNonBlocking));
            cudaGraph_t graph = nullptr;
            CUDA_TRY(cudaStreamBeginCapture(capture_stream, cudaStreamCaptureModeThreadLocal));
            int kernels = 0;
            cudaError_t le = launch_batch(db, tile, sl.seq_flags, capture_stream, &kernels, nullptr);
            sl.graph_kernels[tile_index(tile)][sl.seq_flags] = kernels;
            cudaError_t ce = cudaStreamEndCapture(capture_stream, &graph);
            CUDA_TRY(le);
            CUDA_TRY(ce);
            cudaError_t ie = cudaGraphInstantiate(&g, graph, 0);
            cudaGraphDestroy(graph);
            CUDA_TRY(ie);
        }
        CUDA_TRY(cudaGraphLaunch(g, stream));
        if (launches)
            *launches += sl.graph_kernels[tile_index(tile)][sl.seq_flags];
    } else {
        CUDA_TRY(launch_batch(db, tile, sl.seq_flags, stream, launches, prof));
    }
    keys_dirty = sl.keep_keys;
    unsigned long long *hc = (unsigned long long *)sl.h_counters.ptr; // per-item counters only
    CUDA_TRY(cudaMemcpyAsync(hc + kCounterWords, sl.d_item_counters.ptr,
                             2 * sizeof(unsigned long long) * sl.n_items, cudaMemcpyDeviceToHost, stream));
    if (sl.seq_flags & kSeqLayers) // and the fragment count of a layered view
        CUDA_TRY(cudaMemcpyAsync(hc + C_FRAGS / 2, (unsigned long long *)sl.d_counters.ptr + C_FRAGS / 2,
                                 sizeof(unsigned long long), cudaMemcpyDeviceToHost, stream));
    CUDA_TRY(cudaEventRecord(sl.done, stream));
    return SGL_OK;
}

sgl_status Lane::read_counters(Ctx *ctx, int si, unsigned long long *drawn, unsigned long long *fragments,
                               std::vector<unsigned long long> *per_item)
{
    Slot &sl = slots[si];
    CUDA_TRY(cudaEventSynchronize(sl.done));
    const unsigned long long *hc = (const unsigned long long *)sl.h_counters.ptr;
    const unsigned long long *ic = hc + kCounterWords; // per item: drawn, fragments
    unsigned long long d = 0, f = 0;
    for (int i = 0; i < sl.n_items; i++) {
        d += ic[2 * i];
        f += ic[2 * i + 1];
    }
    if (drawn)
        *drawn = d;
    if (fragments)
        *fragments = f;
    if (per_item)
        per_item->assign(hc + kCounterWords, hc + kCounterWords + 2 * sl.n_items);
    return SGL_OK;
}

sgl_status Lane::layered_fit(Ctx *ctx, int si, bool *fit)
{
    Slot &sl = slots[si];
    CUDA_TRY(cudaEventSynchronize(sl.done));
    const unsigned long long need = ((const unsigned long long *)sl.h_counters.ptr)[C_FRAGS / 2];
    const size_t cap = std::min<size_t>(frags.bytes / sizeof(Frag), 0xFFFFFFFFu);
    *fit = need <= cap;
    if (!*fit) {
        if (need + need / 4 >= 0xFFFFFFFFull) {
            ctx->fail("%llu fragments exceed the fragment pool's 32-bit index", need);
            return SGL_ERR_UNSUPPORTED;
        }
        frag_want = (size_t)(need + need / 4);
    }
    return SGL_OK;
}

} // namespace sgl
