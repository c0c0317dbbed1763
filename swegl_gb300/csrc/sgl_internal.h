// sgl_internal.h — structures shared by the host runtime and the kernels.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace sgl {

constexpr int kMaxPointLights = 16;
constexpr unsigned long long kEmptyKey = ~0ull;     // no fragment won this pixel
constexpr uint32_t kMaxZBits = 0x7F7F7F7Fu;         // viewport_t::clear depth (viewport.cpp:107)

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
    float4 *wpos;            // v_world
    float4 *wnrm;            // normal_world
    float2 *uv;              // tex_coords
    uint32_t n_vertices;
    uint32_t n_triangles;
    int n_mats;
    int n_texs;
    MatDesc default_mat;
};

struct LightsDev {
    float ambient;
    float sun[3];
    float sun_intensity;
    int n;
    float4 pl[kMaxPointLights]; // x, y, z, intensity
};

struct ViewDev {
    int x, y, w, h;
    float view[12];            // rows 0-2 of camera_t::m_viewmatrix
    float proj[12];            // rows 0-2 of camera_t::m_projectionmatrix
    float campos[3];
    float vm00, vm03, vm11, vm13; // viewport_t::m_viewportmatrix (viewport.cpp:94-99)
};

// A span handed from the triangle walk to the long-span kernels: the
// qpixel interpolator of fill_half_triangle after its displacement to x1.
struct SpanRec {
    uint32_t slot;
    uint32_t y_bits;      // y | kBitLower | kBitLLR
    int x1, x2;
    float top, tstep, bottom, bstep, v0, dv;
    float progL, progR;   // edge progress of the row (prepare_for_scanline)
};
static_assert(sizeof(SpanRec) == 48, "SpanRec layout");

constexpr uint32_t kBitLower = 1u << 30; // span of the lower half-triangle
constexpr uint32_t kBitLLR = 1u << 31;   // long_line_on_right
constexpr uint32_t kYMask = (1u << 30) - 1u;
constexpr int kInlineSpan = 16;          // wider spans go to the span queue

// frame counters: 64-bit words [C_DRAWN], [C_FRAGMENTS]; 32-bit words after them
enum { C_DRAWN = 0, C_FRAGMENTS = 1 };
constexpr int kClasses = 5;     // drawable triangles by rows: <=2, <=4, <=8, <=kTallRows, tall
constexpr int kTallRows = 16;   // taller triangles queue every span
enum { C_CLIPTRI = 4, C_SPANS = 5, C_OVERFLOW = 6, C_CLIPPX = 7, C_CLASS0 = 8 };
constexpr int kCounterWords = 8; // 64-bit words (16 32-bit words: C_CLASS0 + kClasses <= 16)

struct FrameDev {
    float4 *ndc;                  // per vertex: v_viewport before the viewport transform
    uint8_t *yes;                 // per vertex visibility flag (mesh_vertex_t::yes)
    unsigned long long *key;      // per view pixel: (depth bits << 32) | draw slot
    float4 *prec;                 // per view pixel: winner's (progress, progL, progR, bits)
    uint32_t *classes;            // drawable triangles in front of the near plane, kClasses lists of n_triangles
    uint32_t *cliptri;            // drawable triangles crossing the near plane (capacity n_triangles)
    uint32_t *clippx;             // pixels won by near-clipped triangles (capacity w*h)
    SpanRec *spans;               // long-span queue
    uint32_t span_cap;
    uint32_t *pixels;             // surface (device), BGRA8, at the viewport's top-left pixel
    int pitch_px;                 // surface row pitch in pixels
    float *zbuf;                  // view w*h depth (may be null)
    unsigned long long *counters; // kCounterWords words
    uint32_t *counters32;         // the same memory seen as 32-bit words
    uint8_t *slot_flags;          // debug: slot reached scanline setup (may be null)
};

// Optional per-kernel timing: CUDA events recorded on the launching stream
// around each kernel of a frame (enabled with sgl_profile).
constexpr int kProfKernels = 9;
enum ProfKernel {
    PK_CLEAR = 0, PK_VERTEX, PK_FLAGS, PK_COMPACT, PK_WALK_DEPTH, PK_SPANS_DEPTH, PK_WALK_WINNER,
    PK_SPANS_WINNER, PK_SHADE
};
struct Profiler {
    bool enabled = false;
    cudaEvent_t ev[kProfKernels + 1] = {};
    double ms[kProfKernels] = {};
    uint64_t launches[kProfKernels] = {};
    bool pending = false;
};
const char *prof_kernel_name(int k);
void prof_flush(Profiler *p);

// kernel launchers (raster.cu)
cudaError_t launch_world(const SceneDev &s, cudaStream_t st);
cudaError_t launch_frame(const SceneDev &s, const LightsDev &l, const ViewDev &v, const FrameDev &f, cudaStream_t st,
                         int *launches, Profiler *prof);

} // namespace sgl
