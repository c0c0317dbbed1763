// sgl_cull.h — the fused geometry pass's whole-primitive frustum test: the
// per-view planes (built on the host with each view's descriptor) and the
// test of a primitive's box against them (run by the kernel, and by the host
// check of the arithmetic).
#pragma once

#include <cmath>
#include <cuda_runtime.h>

#include "sgl.h"

namespace sgl {

// The planes of ViewDev::cull.  The vertex transform computes x' (and y', z')
// as projection row . (view rows . (w, 1), 1) in float, with an error below
// 16 ulp of E(|w|) = |P| . (|V| . |w| + |Vt|) + |Pt| for its row; the bound
// taken is 2^-16 E, so a box that passes the test keeps every vertex at
// least 2^-17 E inside the region (x'/|z'| then rounds strictly past +-1).
inline void cull_planes(const sgl_view &v, float4 cull[5][2])
{
    double M[3][4], E[3][4];
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 4; c++) {
            double m = c == 3 ? (double)v.proj[4 * r + 3] : 0.0, e = c == 3 ? std::fabs((double)v.proj[4 * r + 3]) : 0.0;
            for (int k = 0; k < 3; k++) {
                m += (double)v.proj[4 * r + k] * (double)v.view[4 * k + c];
                e += std::fabs((double)v.proj[4 * r + k]) * std::fabs((double)v.view[4 * k + c]);
            }
            M[r][c] = m;
            E[r][c] = e;
        }
    // a . (w, 1) < 0 where x' < -z', x' > z', y' < -z', y' > z'; and where z' > 0
    const double sx[5] = {1.0, -1.0, 0.0, 0.0, 0.0}, sy[5] = {0.0, 0.0, 1.0, -1.0, 0.0};
    const double sz[5] = {1.0, 1.0, 1.0, 1.0, -1.0};
    for (int p = 0; p < 5; p++) {
        float a[4], e[4];
        for (int c = 0; c < 4; c++) {
            a[c] = (float)(sx[p] * M[0][c] + sy[p] * M[1][c] + sz[p] * M[2][c]);
            e[c] = (float)(0x1p-16 * (std::fabs(sx[p]) * E[0][c] + std::fabs(sy[p]) * E[1][c] + E[2][c]));
        }
        cull[p][0] = make_float4(a[0], a[1], a[2], a[3]);
        cull[p][1] = make_float4(e[0], e[1], e[2], e[3]);
    }
}

// Box (centre bc, half extent bh, ba = |bc| + bh) against region r of
// ViewDev::cull (r[0] the plane, r[1] the error bound): negative when the
// whole box is in the region.
__host__ __device__ __forceinline__ float cull_region(const float4 *r, float4 bc, float4 bh, float4 ba)
{
    const float4 a = r[0], e = r[1];
    return (a.x * bc.x + a.y * bc.y + a.z * bc.z + a.w) + (fabsf(a.x) * bh.x + fabsf(a.y) * bh.y + fabsf(a.z) * bh.z) +
           (e.x * ba.x + e.y * ba.y + e.z * ba.z + e.w);
}

// The box of positions lo .. hi as the geometry pass stores it (k_box):
// centre, half extent; NaN centre when empty or not finite (never culled).
__host__ __device__ __forceinline__ void cull_box(float3 lo, float3 hi, float4 &bc, float4 &bh)
{
    bc = make_float4(0.5f * lo.x + 0.5f * hi.x, 0.5f * lo.y + 0.5f * hi.y, 0.5f * lo.z + 0.5f * hi.z, 0.0f);
    bh = make_float4(0.5f * hi.x - 0.5f * lo.x, 0.5f * hi.y - 0.5f * lo.y, 0.5f * hi.z - 0.5f * lo.z, 0.0f);
    if (!(fabsf(bc.x) + bh.x + fabsf(bc.y) + bh.y + fabsf(bc.z) + bh.z < 0x1p100f))
        bc.x = NAN;
}

// True when the box lies in front of the camera (region z' > 0) and beyond
// one of the side planes: no triangle inside it passes inside_camera_frustum.
__host__ __device__ __forceinline__ bool cull_unseen(const float4 cull[5][2], float4 bc, float4 bh)
{
    const float4 ba = make_float4(fabsf(bc.x) + bh.x, fabsf(bc.y) + bh.y, fabsf(bc.z) + bh.z, 0.0f);
    if (!(cull_region(cull[4], bc, bh, ba) < 0.0f))
        return false;
    for (int r = 0; r < 4; r++)
        if (cull_region(cull[r], bc, bh, ba) < 0.0f)
            return true;
    return false;
}

} // namespace sgl
