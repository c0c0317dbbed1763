// Host check of the fused geometry pass's whole-primitive frustum test, built
// from the same header as the kernels and the library (sgl_cull.h): planes
// from cull_planes, boxes from cull_box, the decision from cull_unseen.  For
// seeded views (cameras near and far, aspect ratios from 1:4096 to 4096:1,
// fields of view from 20 to 120 degrees) and boxes placed across and near each
// side of the view volume (from 1e-6 to 10 units of half extent), wherever
// the test skips a box, every sampled vertex of the box transformed as the
// geometry pass transforms it (transform3 by the view rows, then by the
// projection rows; x and y divided by |z'|) has z' > 0 and lies beyond each
// side the test found: x' / |z'| < -1, >= 1, y' / |z'| < -1 or >= 1, so that
// inside_camera_frustum (src/render/renderer.cpp:58-70) rejects every
// triangle of it.  Prints "<boxes> <skipped> <vertices> <violations>".
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>

#include "sgl_cull.h"
#include "sgl_device.cuh"

using namespace sgl;

// Rows of a camera at `eye` looking at `at` (forward to +z of view space, up
// to +y), row-major 4x4.
static void look_at(const double eye[3], const double at[3], float m[16])
{
    double f[3] = {at[0] - eye[0], at[1] - eye[1], at[2] - eye[2]};
    double l = std::sqrt(f[0] * f[0] + f[1] * f[1] + f[2] * f[2]);
    for (double &x : f)
        x /= l;
    double r[3] = {f[1] * 0.0 - f[2] * 1.0, f[2] * 0.0 - f[0] * 0.0, f[0] * 1.0 - f[1] * 0.0}; // f x up
    l = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    if (l < 1e-9) {
        r[0] = 1.0, r[1] = 0.0, r[2] = 0.0, l = 1.0;
    }
    for (double &x : r)
        x /= l;
    const double u[3] = {r[1] * f[2] - r[2] * f[1], r[2] * f[0] - r[0] * f[2], r[0] * f[1] - r[1] * f[0]};
    const double *rows[3] = {r, u, f};
    for (int i = 0; i < 3; i++) {
        m[4 * i + 0] = (float)rows[i][0];
        m[4 * i + 1] = (float)rows[i][1];
        m[4 * i + 2] = (float)rows[i][2];
        m[4 * i + 3] = (float)-(rows[i][0] * eye[0] + rows[i][1] * eye[1] + rows[i][2] * eye[2]);
    }
    m[12] = m[13] = m[14] = 0.0f;
    m[15] = 1.0f;
}

static void projection(double aspect, double fov_deg, double zn, double zf, float p[16])
{
    const double cot = 1.0 / std::tan(fov_deg * 3.14159265358979323846 / 360.0);
    for (int i = 0; i < 16; i++)
        p[i] = 0.0f;
    p[0] = (float)(cot / aspect);
    p[5] = (float)cot;
    p[10] = (float)(zf / (zf - zn));
    p[11] = (float)(-zf * zn / (zf - zn));
    p[14] = 1.0f;
}

int main(int argc, char **argv)
{
    const long n = argc > 1 ? atol(argv[1]) : 100000;
    std::mt19937_64 g(2024);
    std::uniform_real_distribution<double> u(0.0, 1.0);
    long skipped = 0, vertices = 0, bad = 0;
    for (long c = 0; c < n; c++) {
        // the view
        const double dist = std::exp(std::log(0.5) + u(g) * (std::log(80.0) - std::log(0.5)));
        const double th = u(g) * 6.283185307179586, zc = 2.0 * u(g) - 1.0, rxy = std::sqrt(1.0 - zc * zc);
        const double at[3] = {10.0 * u(g) - 5.0, 10.0 * u(g) - 5.0, 10.0 * u(g) - 5.0};
        const double eye[3] = {at[0] + dist * rxy * std::cos(th), at[1] + dist * zc, at[2] + dist * rxy * std::sin(th)};
        const double aspect = std::exp((2.0 * u(g) - 1.0) * std::log(4096.0));
        sgl_view v{};
        look_at(eye, at, v.view);
        projection(aspect, 20.0 + 100.0 * u(g), 0.01 + u(g), 100.0, v.proj);
        float4 cull[5][2];
        cull_planes(v, cull);
        // a box centre in view space near side s (x'/z' or y'/z' = +-1 + d),
        // or anywhere in front and behind
        const int s = (int)(g() % 5);
        const double zv = std::exp(std::log(0.05) + u(g) * (std::log(200.0) - std::log(0.05))) * (u(g) < 0.1 ? -1.0 : 1.0);
        const double zp = (double)v.proj[10] * zv + (double)v.proj[11];
        const double d = (u(g) < 0.5 ? 1e-6 : 1e-2) * (2.0 * u(g) - 1.0) * std::exp(u(g) * 5.0);
        double q[3];
        if (s < 4) {
            const double ndc = (s & 1 ? 1.0 : -1.0) * (1.0 + d);
            const double other = 2.0 * u(g) - 1.0;
            const double cx = s < 2 ? ndc : other, cy = s < 2 ? other : ndc;
            q[0] = cx * std::fabs(zp) / (double)v.proj[0];
            q[1] = cy * std::fabs(zp) / (double)v.proj[5];
        } else {
            q[0] = (4.0 * u(g) - 2.0) * std::fabs(zv);
            q[1] = (4.0 * u(g) - 2.0) * std::fabs(zv);
        }
        q[2] = zv;
        // world point: the view matrix is a rotation R and a translation t, w = R^T (q - t)
        double w[3];
        for (int k = 0; k < 3; k++)
            w[k] = (double)v.view[0 * 4 + k] * (q[0] - v.view[3]) + (double)v.view[1 * 4 + k] * (q[1] - v.view[7]) +
                   (double)v.view[2 * 4 + k] * (q[2] - v.view[11]);
        const double he = std::exp(std::log(1e-6) + u(g) * (std::log(10.0) - std::log(1e-6)));
        float lo[3], hi[3];
        for (int k = 0; k < 3; k++) {
            const double h = he * (0.2 + u(g));
            lo[k] = (float)(w[k] - h);
            hi[k] = (float)(w[k] + h);
        }
        float4 bc, bh;
        cull_box(make_float3(lo[0], lo[1], lo[2]), make_float3(hi[0], hi[1], hi[2]), bc, bh);
        if (!cull_unseen(cull, bc, bh))
            continue;
        skipped++;
        const float4 ba = make_float4(fabsf(bc.x) + bh.x, fabsf(bc.y) + bh.y, fabsf(bc.z) + bh.z, 0.0f);
        bool side[4];
        for (int r = 0; r < 4; r++)
            side[r] = cull_region(cull[r], bc, bh, ba) < 0.0f;
        // the box's corners and points inside it
        for (int k = 0; k < 40; k++) {
            float p[3];
            for (int a = 0; a < 3; a++) {
                if (k < 8)
                    p[a] = (k >> a) & 1 ? hi[a] : lo[a];
                else {
                    float t = (float)((double)lo[a] + u(g) * ((double)hi[a] - (double)lo[a]));
                    p[a] = t < lo[a] ? lo[a] : (t > hi[a] ? hi[a] : t);
                }
            }
            V3 x = transform3(mk3(p[0], p[1], p[2]), v.view);
            x = transform3(x, v.proj);
            if (x.z != 0.0f) {
                x.x = x.x / fabsf(x.z);
                x.y = x.y / fabsf(x.z);
            }
            vertices++;
            bool ok = x.z > 0.0f;
            ok = ok && (!side[0] || x.x < -1.0f) && (!side[1] || !(x.x < 1.0f));
            ok = ok && (!side[2] || x.y < -1.0f) && (!side[3] || !(x.y < 1.0f));
            if (!ok)
                bad++;
        }
    }
    printf("%ld %ld %ld %ld\n", n, skipped, vertices, bad);
    return 0;
}
