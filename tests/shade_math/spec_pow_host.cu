// Host check of sgl::spec_pow (the specular power of the pixel shader, built
// from the same source as the kernels) against the reference's expression,
// (float)pow((double)s, p) (src/render/pixel_shaders.cpp:193).  Prints
// "<samples> <differing> <differing by more than one unit in the last place>"
// for seeded s in (0, 1] (a third of them within 0.05 of 1, where highlights
// are) and p in 1..pmax, skipping results below 1e-30.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <random>

#include "sgl_device.cuh"

int main(int argc, char **argv)
{
    const long n = argc > 1 ? atol(argv[1]) : 1000000;
    const int pmax = argc > 2 ? atoi(argv[2]) : 128;
    std::mt19937_64 g(12345);
    std::uniform_real_distribution<double> u(0.0, 1.0);
    long used = 0, diff = 0, far = 0;
    for (long i = 0; i < n; i++) {
        float s = (float)u(g);
        if (i % 3 == 0)
            s = 1.0f - (float)(u(g) * 0.05);
        const int p = 1 + (int)(g() % (unsigned long long)pmax);
        if (!(s > 0.0f))
            continue;
        const float want = (float)std::pow((double)s, (double)p);
        if (want < 1e-30f)
            continue;
        used++;
        const float got = sgl::spec_pow(s, p);
        if (got != want) {
            diff++;
            if (got != std::nextafter(want, 2.0f) && got != std::nextafter(want, 0.0f))
                far++;
        }
    }
    printf("%ld %ld %ld\n", used, diff, far);
    return 0;
}
