// noalloc.cu — sgl_render_noalloc: the plain renderer for callers that must
// not allocate memory.
//
// Who needs it: code that runs where allocation is not allowed or not safe —
// a real-time frame callback with a fixed memory plan, a host application that
// hands the renderer a pre-sized device buffer and forbids the library from
// growing its footprint, or code that must not take the allocator's implicit
// device-wide synchronisation (cudaMalloc / cudaFree stall every stream).
// Such a caller cannot use sgl_render, whose per-view scratch (depth keys,
// winner records, triangle lists, span bins, descriptors) lives in
// library-owned buffers that grow on demand.
//
// Here all of that scratch comes from one file-scope device array of
// kNoAllocScratchBytes (64 MiB).  Every GPU that loads the library holds it
// until the process exits.  Views whose scratch does not fit are refused with
// SGL_ERR_BUDGET and a message giving the bytes needed.  The call makes no
// cudaMalloc, cudaFree or other allocating call.  Its descriptors are passed
// by value to a one-block kernel that writes them into the array (kernel
// arguments are copied at launch, so no host buffer has to outlive the call).
//
// The array is shared by every call in a CUDA context and keeps the last
// call's contents; each call clears what must start cleared (the counters in
// the descriptor kernel, the depth keys to all ones with cudaMemsetAsync; the
// visibility flags are cleared by the kernels).  Calls that overlap on the
// GPU in one context (on different streams, or from different host threads)
// race on the array: the caller must order them.  Each CUDA context has its
// own copy of the array, so calls in different contexts do not share it.
//
// Set-up: the first call in a context (the device's primary context, or a
// caller's own driver-API context made current) looks up the array's device
// address in that context with cudaGetSymbolAddress — the array's name is
// only a host-side stand-in — and caches it under the context's unique id
// (cuCtxGetId: ids are never reused in a process, so a context created after
// cudaDeviceReset gets a fresh look-up).  Make that first call before any
// stream capture.
#include <cstdint>
#include <cstring>
#include <mutex>

#include <cuda.h>
#include <cuda_runtime.h>

#include "sgl.h"
#include "sgl_internal.h"
#include "sgl_runtime.h"

namespace sgl {

constexpr size_t kNoAllocScratchBytes = 64ull << 20;
constexpr int kNoAllocMaxContexts = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

static std::mutex g_noalloc_mu;
static unsigned long long g_noalloc_ctx_id[kNoAllocMaxContexts]; // 0: free entry
static void *g_noalloc_addr[kNoAllocMaxContexts];
static int g_noalloc_next;

typedef CUresult (*CtxGetCurrentFn)(CUcontext *);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long *);

// The unique id of the current CUDA context (the runtime's current context,
// after cudaSetDevice: the device's primary context unless the caller made
// its own current).  The driver functions are looked up through the runtime,
// so the library does not link the driver library itself.
static cudaError_t current_context_id(unsigned long long *id)
{
    static CtxGetCurrentFn get_current = nullptr;
    static CtxGetIdFn get_id = nullptr;
    if (!get_current || !get_id) {
        void *f0 = nullptr, *f1 = nullptr;
        cudaDriverEntryPointQueryResult q0, q1;
        cudaError_t e = cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f0, 4000, cudaEnableDefault, &q0);
        if (e == cudaSuccess)
            e = cudaGetDriverEntryPointByVersion("cuCtxGetId", &f1, 12000, cudaEnableDefault, &q1);
        if (e != cudaSuccess)
            return e;
        if (q0 != cudaDriverEntryPointSuccess || q1 != cudaDriverEntryPointSuccess || !f0 || !f1)
            return cudaErrorSymbolNotFound;
        get_current = (CtxGetCurrentFn)f0;
        get_id = (CtxGetIdFn)f1;
    }
    CUcontext c = nullptr;
    if (get_current(&c) != CUDA_SUCCESS || !c)
        return cudaErrorDeviceUninitialized;
    if (get_id(c, id) != CUDA_SUCCESS)
        return cudaErrorDeviceUninitialized;
    return cudaSuccess;
}

// The device address of the scratch array in the current context, looked up
// once per context and cached under the context's id.
static cudaError_t noalloc_scratch(unsigned char **out)
{
    std::lock_guard<std::mutex> g(g_noalloc_mu);
    unsigned long long id = 0;
    cudaError_t e = current_context_id(&id);
    if (e != cudaSuccess)
        return e;
    for (int i = 0; i < kNoAllocMaxContexts; i++)
        if (g_noalloc_ctx_id[i] == id) {
            *out = (unsigned char *)g_noalloc_addr[i];
            return cudaSuccess;
        }
    void *p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess)
        return e;
    const int slot = g_noalloc_next; // the oldest entry makes room (its context is looked up again if used)
    g_noalloc_next = (g_noalloc_next + 1) % kNoAllocMaxContexts;
    g_noalloc_ctx_id[slot] = id;
    g_noalloc_addr[slot] = p;
    *out = (unsigned char *)p;
    return cudaSuccess;
}

// The call's descriptors, passed by value: the item, the batch, the prefix
// arrays and the counters to zero.
struct NoAllocBases {
    uint32_t v[20];
};
__global__ void k_noalloc_setup(ItemDev it, BatchDev b, NoAllocBases bases, ItemDev *item_dst, BatchDev *batch_dst,
                                uint32_t *bases_dst, unsigned long long *counters, unsigned long long *item_counters)
{
    const int t = threadIdx.x;
    if (t == 0) {
        *item_dst = it;
        *batch_dst = b;
    }
    if (t < 20)
        bases_dst[t] = bases.v[t];
    for (int i = t; i < kCounterWords; i += blockDim.x)
        counters[i] = 0ull;
    if (t < 2)
        item_counters[t] = 0ull;
}

static size_t up256(size_t x) { return (x + 255) & ~(size_t)255; }

} // namespace sgl

using namespace sgl;

extern "C" {

SGL_API sgl_status sgl_render_noalloc(sgl_ctx *c, int scene_id, const sgl_view *view, const sgl_target *target,
                                      void *stream)
{
    Ctx *ctx = reinterpret_cast<Ctx *>(c);
    if (!ctx || !view || !target)
        return SGL_ERR_INVALID;
    Scene *s = ctx->find(scene_id);
    if (!s) {
        ctx->fail("unknown scene %d", scene_id);
        return SGL_ERR_NOT_FOUND;
    }
    sgl_status r = check_view(ctx, *view, *target);
    if (r == SGL_OK)
        r = reject_layers(ctx, *view);
    if (r != SGL_OK)
        return r;
    if (cudaSetDevice(ctx->device) != cudaSuccess) {
        ctx->fail("cudaSetDevice(%d) failed", ctx->device);
        return SGL_ERR_CUDA;
    }
    const sgl_view &v = *view;
    const size_t px = (size_t)v.w * v.h;
    const size_t nv = s->n_vertices, nt = s->n_triangles;
    const bool dof = v.dof.enabled != 0;
    const int tile = ctx->tile;
    const size_t tiles = (size_t)((v.w + tile - 1) / tile) * (size_t)((v.h + tile - 1) / tile);
    // layout of the scratch array
    size_t off = 0;
    const size_t o_batch = off;
    off += up256(sizeof(BatchDev));
    const size_t o_item = off;
    off += up256(sizeof(ItemDev));
    const size_t o_bases = off;
    off += up256(20 * sizeof(uint32_t));
    const size_t o_counters = off;
    off += up256(kCounterWords * sizeof(unsigned long long));
    const size_t o_item_counters = off;
    off += up256(2 * sizeof(unsigned long long));
    const size_t o_ndc = off;
    off += up256(16 * nv);
    const size_t o_yes = off;
    off += up256(nv);
    const size_t o_key = off;
    off += up256(8 * px);
    const size_t o_prec = off;
    off += up256(16 * px);
    const bool win_list = px >= kWinListMinPixels; // the shade goes through a winner list
    const size_t o_wins = off;
    off += win_list ? up256(8 * px) : 0;
    const size_t o_list = off;
    off += up256(8 * (nt ? nt : 1));
    const size_t o_recs = off;
    off += up256(sizeof(TriRec) * (nt ? nt : 1));
    const size_t o_tall = off;
    off += up256(4 * (nt ? nt : 1));
    const size_t o_dof = off;
    off += dof ? up256(8 * px) : 0;
    const size_t o_spans = off;
    const size_t min_spans = 4096;
    const size_t need = o_spans + min_spans * sizeof(SpanRec);
    if (need > kNoAllocScratchBytes || px >= (1ull << 32) || tiles >= (1ull << 32)) {
        ctx->fail("sgl_render_noalloc: this view of scene %d needs %zu bytes of scratch; the static scratch "
                  "holds %zu bytes (use sgl_render, or a smaller view or scene)",
                  scene_id, need, kNoAllocScratchBytes);
        return SGL_ERR_BUDGET;
    }
    unsigned char *base = nullptr;
    cudaError_t e = noalloc_scratch(&base);
    if (e != cudaSuccess) {
        ctx->fail("sgl_render_noalloc: cudaGetSymbolAddress: %s", cudaGetErrorString(e));
        return SGL_ERR_CUDA;
    }
    const uint32_t span_cap = (uint32_t)((kNoAllocScratchBytes - o_spans) / sizeof(SpanRec));
    ItemDev it{};
    it.s = s->dev;
    it.v = make_view(v);
    it.ndc = (float4 *)(base + o_ndc);
    it.yes = base + o_yes;
    it.key = (unsigned long long *)(base + o_key);
    it.prec = (float4 *)(base + o_prec);
    it.pixels = (uint32_t *)target->pixels + (size_t)v.y * (target->pitch / 4) + v.x;
    it.pitch_px = target->pitch / 4;
    it.zbuf = target->zbuffer;
    it.tiles_x = (v.w + tile - 1) / tile;
    it.tile_base = 0;
    if (dof) {
        const sgl_dof_desc &d = v.dof;
        it.dof = 1;
        it.dof_out = it.pixels;
        it.dof_pitch = it.pitch_px;
        it.pixels = (uint32_t *)(base + o_dof);
        it.pitch_px = v.w;
        it.dof_src = it.pixels;
        it.dof_src_pitch = v.w;
        if (!it.zbuf)
            it.zbuf = (float *)(base + o_dof + 4 * px);
        const float k = d.px_scale > 0.0f ? d.px_scale : (v.proj[5] * (float)v.h) / 2.0f;
        it.dof_focus = d.focus;
        it.dof_ka = k * d.aperture;
        it.dof_rmax = d.max_radius;
        it.p22 = v.proj[10];
        it.p23 = v.proj[11];
        it.dof_halo = dof_halo_of(d.max_radius);
        it.dof_tiles_x = (v.w + kDofTile - 1) / kDofTile;
    }
    const uint32_t dof_tiles =
        dof ? (uint32_t)((v.w + kDofTile - 1) / kDofTile) * (uint32_t)((v.h + kDofTile - 1) / kDofTile) : 0u;
    const bool fused = s->dev.fused != 0;
    const bool split = !fused || s->dev.mixed != 0; // the general passes run (all, or the larger primitives)
    // prefixes of one item (vertices, triangles, pixels, tiles, depth-of-field
    // tiles, the general geometry pass's vertices and triangles), then the
    // fused pass's one group: its chunks, its items, the item
    const uint32_t chunks = fused ? (s->dev.n_prims + kGeomWarps - 1) / kGeomWarps : 0u;
    const NoAllocBases bases = {{0u, (uint32_t)nv,              0u, (uint32_t)nt,
                                 0u, (uint32_t)px,              0u, (uint32_t)tiles,
                                 0u, dof_tiles,                 0u, split ? (uint32_t)nv : 0u,
                                 0u, split ? (uint32_t)nt : 0u, 0u, chunks,
                                 0u, fused ? 1u : 0u,           0u, 0u}};
    BatchDev b{};
    b.items = (const ItemDev *)(base + o_item);
    const uint32_t *bp = (const uint32_t *)(base + o_bases);
    b.tri_base = bp + 2;
    b.px_base = bp + 4;
    b.tile_base = bp + 6;
    b.dof_base = bp + 8;
    b.g_vtx_base = bp + 10;
    b.g_tri_base = bp + 12;
    b.grp_chunk_base = bp + 14;
    b.grp_item_base = bp + 16;
    b.grp_items = bp + 18;
    b.n_groups = fused ? 1 : 0;
    b.total_gvtx = split ? (uint32_t)nv : 0u;
    b.total_gtri = split ? (uint32_t)nt : 0u;
    b.total_chunks = chunks;
    b.n_items = 1;
    b.inline_span = ctx->inline_span;
    b.total_px = (uint32_t)px;
    b.total_tiles = (uint32_t)tiles;
    b.total_dof_tiles = dof_tiles;
    b.list = (uint2 *)(base + o_list);
    b.list_cap = (uint32_t)(nt ? nt : 1);
    b.clip = b.list;
    b.clip_cap = b.list_cap;
    b.recs = (TriRec *)(base + o_recs);
    b.tall = (uint32_t *)(base + o_tall);
    b.keep_keys = 0;
    b.key_pool = (unsigned long long *)(base + o_key);
    b.wins = win_list ? (uint2 *)(base + o_wins) : nullptr;
    b.spans = (SpanRec *)(base + o_spans);
    b.span_cap = span_cap;
    b.counters = (unsigned long long *)(base + o_counters);
    b.item_counters = (unsigned long long *)(base + o_item_counters);
    b.slot_flags = nullptr;
    cudaStream_t st = (cudaStream_t)stream;
    // descriptors by value; the counters start at zero on every call
    k_noalloc_setup<<<1, 256, 0, st>>>(it, b, bases, (ItemDev *)(base + o_item), (BatchDev *)(base + o_batch),
                                       (uint32_t *)(base + o_bases), (unsigned long long *)(base + o_counters),
                                       (unsigned long long *)(base + o_item_counters));
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaMemsetAsync(base + o_key, 0xFF, 8 * px, st)); // kEmptyKey

    const int seq = (dof ? kSeqDof : 0) | (v.shader != SGL_SHADER_PHONG_BILINEAR ? kSeqShaders : 0) |
                    (fused ? kSeqFused : 0) | (split ? kSeqSplit : 0) | (win_list ? kSeqWinList : 0) | kSeqOne;
    CUDA_TRY(launch_batch((const BatchDev *)(base + o_batch), tile, seq, st, nullptr, nullptr));
    return SGL_OK;
}

} // extern "C"
