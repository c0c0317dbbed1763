// Host check of sgl::light_sum (the sun and point-light sum of the pixel
// shader, built from the same header as the kernels) against a plain
// restatement of the reference's loop (src/render/pixel_shaders.cpp:159-205:
// distance, intensity test, normalisation, alignment test, reflection,
// specular power) that takes every light through every step.  light_sum
// skips lights that are clearly behind the surface before their division;
// the two must agree bit for bit.  Inputs are seeded: random surface points,
// normals, cameras and four point lights, and lights placed almost in the
// tangent plane of the surface (the direction's normal component a tiny
// multiple, of either sign, of its tangent component).  Prints
// "<cases> <differing> <lights skipped early> <near-tangent cases>".
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>

#include "sgl_device.cuh"
#include "sgl_internal.h"
#include "sgl_shade.cuh"

using namespace sgl;

static float plain_light_sum(const LightsDev &L, V3 center, V3 normal, V3 camvec, int shininess)
{
    float face_sun = -dot3(normal, mk3(L.sun[0], L.sun[1], L.sun[2]));
    if (face_sun < 0.0f)
        face_sun = 0.0f;
    else
        face_sun = face_sun * L.sun_intensity;
    float dyn = 0.0f;
    for (int l = 0; l < L.n; l++) {
        const float4 pl = L.pl[l];
        V3 ld = sub3(center, mk3(pl.x, pl.y, pl.z));
        const float d2 = ld.x * ld.x + ld.y * ld.y + ld.z * ld.z;
        float diffuse = pl.w / d2;
        if (diffuse < 0.05f)
            continue;
        ld = normalize3(ld);
        const float alignment = -dot3(normal, ld);
        if (alignment < 0.0f)
            continue;
        diffuse = diffuse * alignment;
        const V3 reflection = add3(ld, mul3(normal, alignment * 2.0f));
        float specular = dot3(reflection, camvec);
        if (specular > 0.0f) {
            specular = spec_pow(specular, shininess);
            specular = specular * (float)shininess / 2.0f;
            dyn = dyn + (diffuse + specular / d2);
        } else {
            dyn = dyn + diffuse;
        }
    }
    return L.ambient + face_sun + dyn;
}

static bool behind_early(V3 normal, V3 ld)
{
    const float d2 = ld.x * ld.x + ld.y * ld.y + ld.z * ld.z;
    const float ax = normal.x * ld.x, ay = normal.y * ld.y, az = normal.z * ld.z;
    const float mag = fabsf(ax) + fabsf(ay) + fabsf(az);
    return ax + ay + az > 0x1p-20f * mag && mag > 0x1p-100f && d2 < 0x1p100f;
}

int main(int argc, char **argv)
{
    const long n = argc > 1 ? atol(argv[1]) : 1000000;
    std::mt19937_64 g(2024);
    std::uniform_real_distribution<float> u(-1.0f, 1.0f);
    auto unit = [&]() {
        V3 v;
        do {
            v = mk3(u(g), u(g), u(g));
        } while (v.x * v.x + v.y * v.y + v.z * v.z < 1e-4f);
        return normalize3(v);
    };
    const float eps[] = {0.0f, 1e-8f, -1e-8f, 1e-7f, -1e-7f, 6e-8f, -6e-8f, 1e-6f, -1e-6f, 3e-5f, -3e-5f};
    long diff = 0, early = 0, tangent = 0;
    for (long i = 0; i < n; i++) {
        LightsDev L{};
        L.ambient = 0.1f;
        const V3 sun = unit();
        L.sun[0] = sun.x, L.sun[1] = sun.y, L.sun[2] = sun.z;
        L.sun_intensity = 0.6f;
        L.n = 4;
        const V3 center = mk3(20.0f * u(g), 20.0f * u(g), 20.0f * u(g));
        const V3 normal = unit();
        const V3 camvec = unit();
        const int shin = 8 + (int)(g() % 121);
        for (int l = 0; l < 4; l++) {
            V3 p = mk3(20.0f * u(g), 20.0f * u(g), 20.0f * u(g));
            if (l == 0 && i % 2 == 0) {
                // a light almost in the surface's tangent plane through the point
                V3 t = sub3(unit(), mul3(normal, dot3(unit(), normal)));
                t = mul3(t, 0.5f + 8.0f * fabsf(u(g)));
                const float e = eps[g() % (sizeof(eps) / sizeof(eps[0]))];
                const V3 d = add3(t, mul3(normal, e * sqrtf(dot3(t, t))));
                p = sub3(center, d);
                tangent++;
            }
            L.pl[l] = make_float4(p.x, p.y, p.z, 50.0f);
            early += behind_early(normal, sub3(center, p)) ? 1 : 0;
        }
        const float a = light_sum(L, center, normal, camvec, shin);
        const float b = plain_light_sum(L, center, normal, camvec, shin);
        if (!(a == b || (a != a && b != b)))
            diff++;
    }
    printf("%ld %ld %ld %ld\n", n, diff, early, tangent);
    return 0;
}
