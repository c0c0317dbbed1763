// sgl_runtime.h — host-side runtime objects behind the C ABI.
#pragma once

#include <map>
#include <memory>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "sgl.h"
#include "sgl_internal.h"

namespace sgl {

constexpr int kMaxBatch = 4096; // views per batch

#define CUDA_TRY(expr)                                                                                                 \
    do {                                                                                                               \
        cudaError_t _e = (expr);                                                                                       \
        if (_e != cudaSuccess) {                                                                                       \
            cudaGetLastError(); /* a failed call's error must not surface in a later launch check */                  \
            ctx->fail("%s: %s", #expr, cudaGetErrorString(_e));                                                        \
            return _e == cudaErrorMemoryAllocation ? SGL_ERR_OOM : SGL_ERR_CUDA;                                       \
        }                                                                                                              \
    } while (0)

// A grow-only device allocation.
struct DevBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
    DevBuf() = default;
    DevBuf(const DevBuf &) = delete;
    DevBuf &operator=(const DevBuf &) = delete;
    ~DevBuf();
    cudaError_t ensure(size_t need);
    void release();
};

// A pinned host allocation.
struct HostBuf {
    void *ptr = nullptr;
    size_t bytes = 0;
    HostBuf() = default;
    HostBuf(const HostBuf &) = delete;
    HostBuf &operator=(const HostBuf &) = delete;
    ~HostBuf();
    cudaError_t ensure(size_t need);
};

struct Ctx;

// A scene resident in device memory.
struct Scene {
    DevBuf d_pos_u, d_nrm_v, d_vnode, d_tris, d_prims, d_mats, d_texs, d_texels, d_wpos, d_wnrm, d_uv,
        d_node_world, d_node_rs, d_lights, d_pgeo, d_pshade, d_psmall, d_vsmall, d_pbox;
    SceneDev dev{};
    LightsDev lights{};
    std::vector<sgl_node_desc> nodes;
    uint32_t n_vertices = 0;
    uint32_t n_triangles = 0;
    size_t device_bytes = 0;

    sgl_status upload_desc(Ctx *ctx, const sgl_scene_desc *d);
    sgl_status refresh_nodes(Ctx *ctx);
    sgl_status set_lights(Ctx *ctx, float ambient, const float *sun, float sun_intensity, const sgl_point_light *pl,
                          int n);
};

// One view of a batch on the host side: its scene, camera and device buffers.
struct BatchEntry {
    Scene *scene;
    sgl_view view;
    uint32_t *rect_pixels; // device, at the viewport's top-left pixel
    int pitch_px;
    float *zbuf;           // device, w*h, may be null
    uint32_t *surface = nullptr; // device, the whole surface (row 0, column 0): views with transparency layers
    float4 *wpos = nullptr;      // device: this view's own world positions and normals (a posed request)
    float4 *wnrm = nullptr;
    float4 *pbox = nullptr;            // device: the boxes of its primitives under the pose (fused scenes)
    const float *node_world = nullptr; // device: this view's own node matrices (a posed request)
    const float *node_rs = nullptr;
};

// node_t::get_local_world_matrix composed with the parents (16 floats per
// node: the world matrix, and the scaled rotation that turns normals); false
// for a cycle or a bad parent.
bool node_matrices(const std::vector<sgl_node_desc> &nodes, std::vector<float> &world, std::vector<float> &rs);

// Scratch bytes a view needs beyond its output buffers: vertex NDC and flags,
// per-pixel keys and winner records, and its share of the batch lists.
size_t view_scratch_bytes(uint32_t n_vertices, uint32_t n_triangles, int w, int h);

// A stream with everything a batch launch sequence needs.  Descriptors are
// staged in pinned memory and copied per batch; a ring of staging slots lets
// several batches be queued on the stream.  The device buffers that the
// launch sequence names directly (descriptors, counters) never move, so a
// captured CUDA graph stays valid; the pools they point to may grow.
struct Lane {
    static constexpr int kSlots = 4;
    int max_items = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t capture_stream = nullptr;
    bool own_stream = false;
    struct Slot {
        DevBuf d_items, d_bases, d_batch, d_counters, d_item_counters;
        HostBuf h_items, h_bases, h_batch, h_counters;
        cudaEvent_t staged = nullptr; // staging copies of this slot done
        cudaEvent_t done = nullptr;   // launch sequence of this slot done
        bool used = false;
        cudaGraphExec_t graph[3][kSeqVariants] = {}; // per tile 8/16/32 and sequence flags (kSeq*)
        int graph_kernels[3][kSeqVariants] = {};     // kernels in each graph
        int n_items = 0;
        int seq_flags = 0;
        bool keep_keys = false;
    } slots[kSlots];
    int next = 0;
    DevBuf list, recs, tall, spans, ndc, yes, key, prec, wins, doftmp, dofz;
    DevBuf frags, frag_head, layer0; // views with transparency layers
    DevBuf poses;                    // batch items with their own pose: node matrices, world positions, normals
    static constexpr int kBaseArrays = 10; // prefixes: vertices, triangles, pixels, tiles, dof tiles, the
                                           // general geometry pass's vertices and triangles; the fused
                                           // pass's group chunks, group items and the grouped items
    size_t frag_want = 0;            // fragments the pool must hold (grown after an overflow)
    bool keys_dirty = false; // the key pool may hold other than kEmptyKey (debug, failed launch)
    ~Lane();

    // external == nullptr: own stream, blocking (ordered with the legacy default stream) or not
    sgl_status init(Ctx *ctx, int max_items, cudaStream_t external, bool blocking = false);
    // Stage and copy the descriptors of a batch into a free slot; returns its index.
    sgl_status prepare(Ctx *ctx, const BatchEntry *e, int n, int tile, int inline_span, uint8_t *slot_flags,
                       int *slot_out);
    // Run the launch sequence of a prepared slot (directly, or as a CUDA graph).
    sgl_status launch(Ctx *ctx, int slot, int tile, bool use_graph, int *launches, Profiler *prof);
    // Per-batch and per-item counters of a finished slot (synchronises the slot).
    sgl_status read_counters(Ctx *ctx, int slot, unsigned long long *drawn, unsigned long long *fragments,
                             std::vector<unsigned long long> *per_item);
    // A finished layered slot: true when its fragment pool was big enough,
    // else grows frag_want for the next attempt (synchronises the slot).
    sgl_status layered_fit(Ctx *ctx, int slot, bool *fit);
};

struct Ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::string last_error;
    std::map<int, std::unique_ptr<Scene>> scenes;
    int next_scene_id = 1;
    std::unique_ptr<Lane> lane;        // the plain renderer's lane (internal stream)
    std::unique_ptr<Lane> ext_lane;    // lane bound to caller streams
    DevBuf stage_pixels, stage_z, debug_flags, dof_stage, dof_desc;
    Profiler prof;
    int tile = 16;                     // shade tile of the plain renderer
    int inline_span = 16;              // long-span bin threshold of the plain renderer

    void fail(const char *fmt, ...) __attribute__((format(printf, 2, 3)));
    Scene *find(int id)
    {
        auto it = scenes.find(id);
        return it == scenes.end() ? nullptr : it->second.get();
    }
};

ViewDev make_view(const sgl_view &v);
sgl_status check_view(Ctx *ctx, const sgl_view &v, const sgl_target &t);
sgl_status reject_layers(Ctx *ctx, const sgl_view &v);

} // namespace sgl
