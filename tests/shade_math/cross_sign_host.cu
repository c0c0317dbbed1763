// Host check of sgl::cross_z_positive / cross_z_negative (the back-face and
// front-face tests of the geometry and set-up passes, built from the same
// header as the kernels) against the reference's expression: the z of the
// normalised cross product (cross(), src/projection/points.cpp:32-37; its
// normalize(), swegl/projection/points.hpp:71-90) compared with zero.
// Seeded edge vectors of ordinary, tiny, huge, subnormal, zero, infinite and
// NaN components.  Prints "<cases> <differing>".
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <limits>
#include <random>

#include "sgl_device.cuh"

using namespace sgl;

static float ref_z(V3 a, V3 b)
{
    V3 c = mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
    c = normalize3(c);
    return c.z;
}

int main(int argc, char **argv)
{
    const long n = argc > 1 ? atol(argv[1]) : 1000000;
    std::mt19937_64 g(99);
    std::uniform_real_distribution<float> u(-1.0f, 1.0f);
    const float special[] = {0.0f,     -0.0f,     1e-30f,  -1e-30f, 1e-40f, -1e-40f, 1e-20f, 1e-25f, 3e-27f,
                             1e19f,    -1e19f,    3e25f,   1e30f,   -1e30f, 3e38f,   std::numeric_limits<float>::infinity(),
                             -std::numeric_limits<float>::infinity(), std::numeric_limits<float>::quiet_NaN(),
                             0x1p-80f, -0x1p-80f, 0x1p-81f, 0x1p-64f, 0x1p-75f};
    const int ns = sizeof(special) / sizeof(special[0]);
    auto comp = [&]() {
        const int kind = (int)(g() % 8);
        if (kind == 0)
            return special[g() % ns];
        const float v = u(g);
        if (kind == 1)
            return v * 1e-12f;
        if (kind == 2)
            return v * 1e18f;
        if (kind == 3)
            return v * 1e-30f;
        return v;
    };
    long diff = 0;
    for (long i = 0; i < n; i++) {
        V3 a = mk3(comp(), comp(), comp()), b = mk3(comp(), comp(), comp());
        if (i % 4 == 0) { // nearly parallel edges: a tiny cross product
            const float e = (float)(g() % 1000) * 1e-9f;
            b = mk3(a.x * 2.0f + e, a.y * 2.0f, a.z * 2.0f - e);
        }
        const float z = ref_z(a, b);
        if (cross_z_positive(a, b) != (z > 0.0f) || cross_z_negative(a, b) != (z < 0.0f))
            diff++;
    }
    printf("%ld %ld\n", n, diff);
    return 0;
}
