// sgl_internal.h — structures shared by the host runtime and the kernels.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "sgl.h"

namespace sgl {

constexpr int kMaxPointLights = 16;
constexpr unsigned long long kEmptyKey = ~0ull; // no fragment won this pixel
constexpr uint32_t kMaxZBits = 0x7F7F7F7Fu;     // viewport_t::clear depth (viewport.cpp:107)

struct TexDesc {
    const uint32_t *texels;
    int w, h;
};

struct MatDesc {
    uint32_t color;
    int texture;
    int double_sided;
    int shininess;
};

struct PrimDesc {
    int material;
    int node;
};

// What the pixel shader binds for a primitive, resolved at upload
// (pixel_shader_t::prepare_for_primitive, src/render/pixel_shaders.cpp:14-31,
// 284-302): its material's colour, shininess and texture — or the scene's
// default material when its index is out of range — and, for the visibility
// flags, whether its material is double sided (renderer.cpp:135-150: false
// for an out-of-range index).
struct __align__(16) PrimShade {
    const uint32_t *tex; // mip 0 texels, nullptr when untextured
    int tw, th;          // 1 x 1 when untextured
    uint32_t color;
    int shininess;
    int double_sided;
    int pad;
};
static_assert(sizeof(PrimShade) == 32, "PrimShade layout");

// Scenes whose every primitive has at most kFuseVerts vertices and
// kFuseTris triangles take the fused geometry pass (one warp per primitive:
// vertex transform, visibility flags and compaction in shared memory).
constexpr uint32_t kFuseVerts = 256, kFuseTris = 512;
// The fused geometry pass: a block takes kGeomWarps primitives of a group (one
// warp each) and runs them for every item of the group.
constexpr int kGeomWarps = 8;

struct LightsDev {
    float ambient;
    float sun[3];
    float sun_intensity;
    int n;
    float4 pl[kMaxPointLights]; // x, y, z, intensity
};

// Device-resident scene (all pointers are device memory).
struct SceneDev {
    const float4 *pos_u;     // (x, y, z, u)
    const float4 *nrm_v;     // (nx, ny, nz, v)
    const uint32_t *vnode;   // node of each vertex
    const uint4 *tris;       // draw-order triangles: 3 global vertex indices + draw-order primitive
    const PrimDesc *prims;   // draw-order primitives
    const MatDesc *mats;
    const TexDesc *texs;
    const float *node_world; // 16 floats per node
    const float *node_rs;    // 16 floats per node
    const LightsDev *lights;
    float4 *wpos;            // v_world
    float4 *wnrm;            // normal_world
    float2 *uv;              // tex_coords
    const uint4 *pgeo;       // draw-order primitives: first vertex, vertex count, first triangle, triangle count
    const PrimShade *pshade; // draw-order primitives: material and texture as the pixel shader binds them
    uint32_t n_vertices;
    uint32_t n_triangles;
    uint32_t n_prims;
    int fused;               // some primitive within kFuseVerts / kFuseTris: the fused geometry pass runs
    int mixed;               // fused, and some primitive beyond the limits: the general passes run too
    const uint8_t *psmall;   // mixed: per draw-order primitive, 1 when the fused pass takes it
    const uint8_t *vsmall;   // mixed: per vertex, 1 when only primitives of the fused pass use it
    float4 *pbox;            // fused: per draw-order primitive, the centre then the half extent of the box of its
                             // world positions (k_box, after k_world); the fused pass's whole-primitive frustum test
    int n_mats;
    int n_texs;
    MatDesc default_mat;
};

struct ViewDev {
    int x, y, w, h;
    float view[12];               // rows 0-2 of camera_t::m_viewmatrix
    float proj[12];               // rows 0-2 of camera_t::m_projectionmatrix
    float campos[3];
    float vm00, vm03, vm11, vm13; // viewport_t::m_viewportmatrix (viewport.cpp:94-99)
    int shader;                   // SGL_SHADER_* (include/sgl.h)
    // Whole-primitive frustum test (make_view): for each of the regions
    // x' < -z', x' > z', y' < -z', y' > z' and z' > 0 of the projected
    // coordinates, a world-space plane a (negative in the region) and an
    // error bound e (>= 0), as cull[r][0] = a and cull[r][1] = e.  Over a box
    // with centre C and half extent H, a negative a.C + a3 + |a|.H +
    // e.(|C| + H) + e3 puts every point of the box in the region by far more
    // than the rounding of the vertex transform; a box in one of the first
    // four regions and in the fifth holds no triangle that
    // inside_camera_frustum accepts.
    float4 cull[5][2];
};

// One view of a batch: its scene, camera and buffers.
struct ItemDev {
    SceneDev s;
    ViewDev v;
    float4 *ndc;             // per vertex: v_viewport before the viewport transform
    uint8_t *yes;            // per vertex: kYesDrawn (mesh_vertex_t::yes) | kYesBehind (z' below the near plane)
    unsigned long long *key; // per view pixel: (depth bits << 32) | draw slot
    float4 *prec;            // per view pixel: recorded winner (progress, progL, progR, bits)
    uint32_t *pixels;        // surface (device), BGRA8, at the viewport's top-left pixel
    int pitch_px;            // surface row pitch in pixels
    float *zbuf;             // view w*h depth (may be null)
    int tiles_x;             // shade tiles across the view
    uint32_t tile_base;      // first shade tile of this item in the batch
    // depth-of-field gather (when dof != 0 the shade kernel writes `pixels`
    // as a scratch colour buffer of pitch w, and the gather writes dof_out)
    int dof;
    float dof_focus, dof_ka, dof_rmax, p22, p23;
    uint32_t *dof_out;
    int dof_pitch;
    uint32_t *dof_src;  // the gather's colour input (pitch dof_src_pitch): the shade's scratch buffer, or for a
    int dof_src_pitch;  // view with transparency layers a copy of its rectangle after the layer passes
    int dof_halo;    // tap reach in pixels (ceil of max_radius, <= kDofMaxHalo), -1: gather from memory
    int dof_tiles_x; // kDofTile tiles across the view
    // transparency layers (viewport_t::m_transparency_layers); when layers
    // > 0, `pixels` points into a whole surface whose row 0, column 0 is
    // `surface`, and each view pixel has a fragment list and a layer colour
    int layers;
    uint32_t *surface;
    uint32_t *frag_head; // per view pixel: first fragment (kFragEnd: none)
    uint32_t *layer0;    // per view pixel: the layers merged into the first one
};

// One fragment of a view with transparency layers: its depth, draw slot and
// the progress values that shade it, chained per pixel.
struct __align__(16) Frag {
    float4 rec;   // progress, progL, progR, span bits (as in ItemDev::prec)
    uint32_t z;   // depth bits
    uint32_t slot;
    uint32_t next; // the next fragment of the pixel; before linking, the view pixel (kFragEnd: a hole)
    uint32_t pad;
};
static_assert(sizeof(Frag) == 32 && offsetof(Frag, next) == 24, "Frag layout");
constexpr uint32_t kFragEnd = 0xFFFFFFFFu;

constexpr uint8_t kYesDrawn = 1;  // a visible triangle flagged the vertex (renderer.cpp:86-185)
constexpr uint8_t kYesBehind = 2; // its z' is below the near plane (fill_triangle's clip test)

// Depth-of-field tiles: kDofTile x kDofTile pixels with a halo of up to
// kDofMaxHalo pixels staged in shared memory.
constexpr int kDofTile = 32;
constexpr int kDofMaxHalo = 32;
// Row pitch of the staged tile in shared memory, the same for every halo so
// that the rows of a tap are constant offsets apart.
constexpr int kDofPitch = kDofTile + 2 * kDofMaxHalo;

// The tap reach of a depth-of-field view: ceil(max_radius) when it fits the
// staged halo, else -1 (the gather then reads the colour buffer directly).
inline int dof_halo_of(float max_radius)
{
    if (!(max_radius >= 0.0f && max_radius <= (float)kDofMaxHalo))
        return -1;
    int h = (int)max_radius;
    if ((float)h < max_radius)
        h++;
    return h;
}

// A span handed from the triangle walk to the long-span kernels: the qpixel
// interpolator of fill_half_triangle after its displacement to x1.
struct SpanRec {
    uint32_t slot;
    uint32_t y_bits; // y | kBitLower | kBitLLR
    int x1, x2;
    float top, tstep, bottom, bstep, v0, dv;
    float progL, progR; // edge progress of the row (prepare_for_scanline)
    uint32_t item;
};
static_assert(sizeof(SpanRec) == 52, "SpanRec layout");

constexpr uint32_t kBitLower = 1u << 30; // span of the lower half-triangle
constexpr uint32_t kBitLLR = 1u << 31;   // long_line_on_right
constexpr uint32_t kYMask = (1u << 30) - 1u;
constexpr int kTallRows = 16; // triangles walking more rows bin every span

// The scanline set-up of one drawable triangle (fill_triangle_2,
// src/render/renderer.cpp:361-460), written by the walk and read back by the
// shade kernel, which replays a winner's row and pixel steps from it instead
// of repeating the set-up.  Vertices are in fill_triangle_2's y order
// (v0, v1, v2).  Each edge is an interpolator_g<1> with its x, after the
// displacement to the first row the walk visits: the long edge v0 -> v2 and
// the upper short edge v0 -> v1 at row y_s, the lower short edge v1 -> v2 at
// row y_l.  Row k of the walk (k < n_u: upper half, else lower half) sees the
// long edge after k steps and its short edge after k (or k - n_u) steps.
struct __align__(16) TriRec {
    float lx, ltop, lbot, lratio;  // long edge
    float ltstep, lbstep, ux, utop; // ... upper short edge
    float ubot, uratio, utstep, ubstep;
    float dx, dtop, dbot, dratio;   // lower short edge
    float dtstep, dbstep, z0, z1;   // z' of v0, v1, v2
    float z2;
    int y_s, y_l, n_u;
    int n_d;
    uint32_t flags;                 // kRecLLRUpper | kRecLLRLower | kRecFFV | kRecTall
    uint32_t slot, item;
    uint32_t g0, g1, g2, prim;      // vertices of v0, v1, v2; draw-order primitive
};
static_assert(sizeof(TriRec) == 128, "TriRec layout");
constexpr uint32_t kRecLLRUpper = 1u; // long_line_on_right in the upper half
constexpr uint32_t kRecLLRLower = 2u; // ... in the lower half
constexpr uint32_t kRecFFV = 4u;      // front_face_visible
constexpr uint32_t kRecTall = 8u;     // every span was binned (winners recorded in prec)
// The flags word of the record slot of a near-clipped triangle (written by the
// geometry passes; such a triangle gets no set-up record).
constexpr uint32_t kRecClip = 0xFFFFFFFFu;
constexpr int kRecFlagsWord = 25; // 32-bit word of TriRec::flags
static_assert(offsetof(TriRec, flags) == 4 * kRecFlagsWord, "TriRec::flags word");

// Batch counters (32-bit words); the drawn-triangle and fragment counts are
// kept per item (item_counters) and summed by the host.
enum { C_LIST = 4, C_CLIP = 5, C_SPANS = 6, C_OVERFLOW = 7, C_FRAGS = 8, C_TALL = 10, C_WINS = 12, C_DOF_NEXT = 14 };
// Work queues of the shade kernel's tiles: kQueues counters, one per 128-byte
// line so that blocks of different queues do not contend.
constexpr int kQueues = 16;
constexpr int C_SHADE_Q = 32;                       // 32-bit index of queue q: C_SHADE_Q + 32 q
constexpr int kCounterWords = (C_SHADE_Q + 32 * kQueues) / 2; // 64-bit words

// A batch of views rendered by one launch sequence (lives in device memory).
struct BatchDev {
    const ItemDev *items;
    const uint32_t *tri_base;  // n_items + 1 prefix of triangle counts
    const uint32_t *px_base;   // n_items + 1 prefix of pixel counts
    const uint32_t *tile_base; // n_items + 1 prefix of shade-tile counts
    const uint32_t *dof_base;  // n_items + 1 prefix of depth-of-field tile counts (0 for items without)
    // the geometry passes: items of fused scenes in groups that read the same
    // vertex data (one scene, or one posed request's own world positions) —
    // group g holds the items grp_items[grp_item_base[g] .. grp_item_base[g+1])
    // and the chunks grp_chunk_base[g] .. grp_chunk_base[g+1] of kGeomWarps
    // primitives each; the other items by vertex and triangle (g_vtx_base,
    // g_tri_base).  Each item counts in one of the two.
    const uint32_t *g_vtx_base, *g_tri_base;
    const uint32_t *grp_chunk_base, *grp_item_base, *grp_items;
    uint32_t total_gvtx, total_gtri, total_chunks;
    int n_groups;
    int n_items;
    int inline_span;           // spans wider than this go to the long-span bins
    uint32_t total_px, total_tiles, total_dof_tiles;
    uint2 *list;               // drawable triangles {batch triangle (tri_base[item] + t), item}
    uint32_t list_cap;
    uint2 *clip;               // drawable triangles crossing the near plane {t, item}: entry j at clip[clip_cap - 1 - j]
    uint32_t clip_cap;
    TriRec *recs;              // per batch triangle (tri_base[item] + t): the scanline set-up of a walk-list
                               // triangle, or flags kRecClip for a near-clipped one (others: stale)
    uint32_t *tall;            // batch triangles of the tall set-ups (list_cap entries)
    int keep_keys;             // leave the depth keys for the caller (debug); else the shade resets them
    unsigned long long *key_pool; // the items' depth keys: batch pixel px_base[item] + i at key_pool[...]
    uint2 *wins;               // kSeqWinList: pixels with a winner {batch pixel, draw slot}, in pixel order
    SpanRec *spans;            // long-span bins
    uint32_t span_cap;
    unsigned long long *counters;      // kCounterWords words
    unsigned long long *item_counters; // per item: drawn, fragments
    uint8_t *slot_flags;       // debug, single-item batches: slot reached scanline setup
    Frag *frags;               // fragment pool of the views with transparency layers
    uint32_t frag_cap;
};

// Optional per-kernel timing: CUDA events recorded on the launching stream
// around each stage of a launch sequence (enabled with sgl_profile).
constexpr int kProfKernels = 14;
enum ProfKernel {
    PK_GEOM = 0, PK_VERTEX, PK_FLAGS, PK_COMPACT, PK_SETUP, PK_WALK, PK_SPANS, PK_WINNER, PK_SHADE, PK_DOF,
    PK_FRAGS, PK_LAYERS, PK_FLATTEN, PK_COPY
};
struct Profiler {
    bool enabled = false;
    cudaEvent_t ev[kProfKernels + 1] = {};
    double ms[kProfKernels] = {};
    uint64_t launches[kProfKernels] = {};
    uint32_t ran = 0; // stages the pending sequence launched (bit per ProfKernel)
    bool pending = false;
};
const char *prof_kernel_name(int k);
void prof_flush(Profiler *p);

// kernel launchers (raster.cu)
cudaError_t launch_world(const SceneDev &s, cudaStream_t st);
// The world positions and normals of a scene under other node matrices
// (`node_world`, `node_rs`, device) into `wpos` / `wnrm` (a posed request),
// and the boxes of its primitives into `pbox` (2 float4 per primitive, may
// be null); the scene's own arrays are not touched.
cudaError_t launch_pose(const SceneDev &s, const float *node_world, const float *node_rs, float4 *wpos, float4 *wnrm,
                        float4 *pbox, cudaStream_t st);
// The launch sequence of a batch whose BatchDev lives at `b` (device memory).
// `flags`: kSeqDof adds the depth-of-field gather, kSeqShaders shades with
// every pixel shader (a view asks for another than the default).  The depth
// keys must hold
// kEmptyKey on entry; the shade kernel leaves them so (unless keep_keys).
// kSeqLayers (a single view with transparency layers) replaces the depth walk
// and shade by the fragment capture, the per-pixel layer resolve and the
// flatten and copy passes; its fragment pool must have been big enough
// (C_FRAGS <= frag_cap) for the outputs to be written, else they are left
// untouched and the host renders again with a bigger pool.
// kSeqFused: items of fused scenes (k_geom); kSeqSplit: other items (k_vertex,
// k_flags, k_compact).  kSeqWinList shades through a winner list (k_classify
// then k_shade_wins, for a batch of one large view) instead of the tiled
// k_shade; BatchDev::wins must then hold total_px entries.  kSeqOne: the
// batch has one view (the walk deals its list entries strided over groups).
constexpr int kSeqDof = 1, kSeqShaders = 2, kSeqLayers = 4, kSeqFused = 8, kSeqSplit = 16, kSeqWinList = 32,
              kSeqOne = 64, kSeqVariants = 128;
// A batch of one view of at least this many pixels shades through the winner
// list: the tiled shade's per-tile key reads and barriers then cost more than
// the list's second kernel and its round trip through L2.
constexpr uint64_t kWinListMinPixels = 1u << 20;
cudaError_t launch_batch(const BatchDev *b, int tile, int flags, cudaStream_t st, int *launches, Profiler *prof);
// The device-side bounds checks of the checked build (-DSGL_BOUNDS_CHECK):
// the first failure's check code and index and the failure count, cleared
// when `reset`; `compiled` says whether this build has the checks.
cudaError_t check_status(unsigned *code, unsigned long long *index, unsigned *count, bool reset, bool *compiled);
// The depth-of-field gather alone (items prepared by the caller).
cudaError_t launch_dof(const BatchDev *b, cudaStream_t st);
// Upload the constant tables (depth-of-field taps) to the current device and
// set the kernels' shared-memory limits there; before any launch or capture.
cudaError_t init_device_constants();

} // namespace sgl
