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

struct FrameDev {
    float4 *ndc;                  // per vertex: v_viewport before the viewport transform
    uint8_t *yes;                 // per vertex visibility flag (mesh_vertex_t::yes)
    unsigned long long *key;      // per view pixel: (depth bits << 32) | draw slot
    uint32_t *pixels;             // surface (device), BGRA8, at the viewport's top-left pixel
    int pitch_px;                 // surface row pitch in pixels
    float *zbuf;                  // view w*h depth
    unsigned long long *counters; // [0] drawn (sub-)triangles, [1] fragments
    uint8_t *slot_flags;          // debug: slot reached scanline setup (may be null)
};

// kernel launchers (raster.cu)
cudaError_t launch_world(const SceneDev &s, cudaStream_t st);
cudaError_t launch_frame(const SceneDev &s, const LightsDev &l, const ViewDev &v, const FrameDev &f, cudaStream_t st,
                         int *launches);

} // namespace sgl
