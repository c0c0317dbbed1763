// sgl_device.cuh — device-side arithmetic of the swegl render path.
//
// Every helper performs the same IEEE single-precision operations, in the same
// order, as the reference function cited beside it (paths inside
// gbizzotto/swegl), so that coverage, depth and the depth-test winner are
// bit-exact.  The library is compiled with -fmad=false (no fused
// multiply-add contraction), IEEE division and square root (no fast-math) and
// denormals preserved, matching the reference's x86-64 SSE build.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace sgl {

// Device-side bounds checks.  The checked build (-DSGL_BOUNDS_CHECK, the
// library libsgl_check.so) tests the index of each guarded access against its
// buffer; an index outside records its check code and the index in a status
// word (the first failure, and a count) and the access is skipped: nothing
// traps and no kernel waits.  The host reads the status with
// sgl_check_status().  In the normal build the checks compile away.
enum CheckCode : unsigned {
    CHK_NDC = 1,      // projected vertex: index against the scene's vertices
    CHK_REC = 2,      // set-up record slot: batch triangle against the record pool
    CHK_KEY = 3,      // depth key: pixel against the view rectangle
    CHK_PREC = 4,     // winner record: pixel against the view
    CHK_PIXEL = 5,    // output colour / depth: pixel against the view
    CHK_TEXEL = 6,    // texel against its texture
    CHK_LOCAL = 7,    // local vertex index of a fused primitive against its vertex count
    CHK_DOF = 8,      // depth-of-field output: pixel against the view
};
#ifdef SGL_BOUNDS_CHECK
static __device__ unsigned long long g_check_first; // code << 48 | index (low 48 bits); 0: no failure
static __device__ unsigned int g_check_count;
__device__ __forceinline__ bool in_bounds(bool ok, unsigned code, unsigned long long index)
{
    if (!ok) {
        atomicCAS(&g_check_first, 0ull, ((unsigned long long)code << 48) | (index & 0xFFFFFFFFFFFFull));
        atomicAdd(&g_check_count, 1u);
    }
    return ok;
}
#else
__device__ __forceinline__ constexpr bool in_bounds(bool, unsigned, unsigned long long) { return true; }
#endif

struct V3 {
    float x, y, z;
};
struct V2 {
    float x, y;
};

__host__ __device__ __forceinline__ V3 mk3(float x, float y, float z) { return V3{x, y, z}; }
__host__ __device__ __forceinline__ V3 add3(V3 a, V3 b) { return mk3(a.x + b.x, a.y + b.y, a.z + b.z); }
__host__ __device__ __forceinline__ V3 sub3(V3 a, V3 b) { return mk3(a.x - b.x, a.y - b.y, a.z - b.z); }
__host__ __device__ __forceinline__ V3 mul3(V3 a, float s) { return mk3(a.x * s, a.y * s, a.z * s); }
__host__ __device__ __forceinline__ V3 neg3(V3 a) { return mk3(-a.x, -a.y, -a.z); }
// vector_t::dot (swegl/projection/points.hpp:91-94)
__host__ __device__ __forceinline__ float dot3(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V2 mk2(float x, float y) { return V2{x, y}; }
__device__ __forceinline__ V2 add2(V2 a, V2 b) { return mk2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ V2 sub2(V2 a, V2 b) { return mk2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ V2 mul2(V2 a, float s) { return mk2(a.x * s, a.y * s); }

// vector_t::normalize (swegl/projection/points.hpp:71-90)
__host__ __device__ __forceinline__ V3 normalize3(V3 v)
{
    float l = sqrtf(v.x * v.x + v.y * v.y + v.z * v.z);
    if (l != 0.0f) {
        v.x = v.x / l;
        v.y = v.y / l;
        v.z = v.z / l;
    }
    return v;
}

// cross() returns a normalised normal_t (src/projection/points.cpp:32-37)
__device__ __forceinline__ V3 cross_n(V3 a, V3 b)
{
    return normalize3(mk3(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x));
}

// cross(a, b).z() > 0 for the normalised cross product (points.cpp:32-37;
// front_face_visible, renderer.cpp:72-75): normalize() divides each
// component by the same length l = sqrt(x^2 + y^2 + z^2), so only z / l is
// needed, and only its sign.  z <= 0 (or NaN) gives z / l <= 0 (or NaN).
// For z >= 2^-80 with a finite sum of squares, l is at most sqrt(FLT_MAX) <
// 2^64, so z / l >= 2^-144 rounds to a positive float (or l = 0, and
// normalize() leaves z, positive); only smaller z or an infinite or NaN sum
// take the reference's expression.
__host__ __device__ __forceinline__ bool cross_z_positive(V3 a, V3 b)
{
    const float x = a.y * b.z - a.z * b.y, y = a.z * b.x - a.x * b.z, z = a.x * b.y - a.y * b.x;
    if (!(z > 0.0f))
        return false;
    const float s = x * x + y * y + z * z;
    if (z >= 0x1p-80f && s <= 3.40282347e38f)
        return true;
    const float l = sqrtf(s);
    return (l != 0.0f ? z / l : z) > 0.0f;
}
// cross(a, b).z() < 0 for the normalised cross product, by the same argument.
__host__ __device__ __forceinline__ bool cross_z_negative(V3 a, V3 b)
{
    const float x = a.y * b.z - a.z * b.y, y = a.z * b.x - a.x * b.z, z = a.x * b.y - a.y * b.x;
    if (!(z < 0.0f))
        return false;
    const float s = x * x + y * y + z * z;
    if (z <= -0x1p-80f && s <= 3.40282347e38f)
        return true;
    const float l = sqrtf(s);
    return (l != 0.0f ? z / l : z) < 0.0f;
}

// transform(vertex, m): rows 0-2 only (src/projection/points.cpp:8-13)
__host__ __device__ __forceinline__ V3 transform3(V3 v, const float *m)
{
    return mk3(m[0] * v.x + m[1] * v.y + m[2] * v.z + m[3], m[4] * v.x + m[5] * v.y + m[6] * v.z + m[7],
               m[8] * v.x + m[9] * v.y + m[10] * v.z + m[11]);
}

// rotate(normal, m) then the normal_t constructor (src/projection/points.cpp:44-49)
__device__ __forceinline__ V3 rotate_n(V3 v, const float *m)
{
    return normalize3(mk3(m[0] * v.x + m[1] * v.y + m[2] * v.z, m[4] * v.x + m[5] * v.y + m[6] * v.z,
                          m[8] * v.x + m[9] * v.y + m[10] * v.z));
}

// (int)f as the reference's x86-64 build evaluates it (cvttss2si): out of
// range and NaN give INT_MIN.  The hardware conversion saturates instead.
__device__ __forceinline__ int f2i(float f)
{
    return (f >= -2147483648.0f && f < 2147483648.0f) ? __float2int_rz(f) : INT32_MIN;
}

// The reference compares floats with the double constants 0.001 and 0.05
// (renderer.cpp:65,281,286,489; pixel_shaders.cpp:179).  0.001f and 0.05f are
// the smallest floats above those doubles, so for a float x:
//   (double)x <  0.001  <=>  x <  0.001f      (double)x >= 0.001  <=>  x >= 0.001f
//   (double)x <= 0.001  <=>  x <  0.001f      (double)x <  0.05   <=>  x <  0.05f
// which keeps these tests off the FP64 pipe.
__device__ __forceinline__ bool below_near(float x) { return x < 0.001f; }    // (double)x < 0.001, or <= 0.001
__device__ __forceinline__ bool at_or_past_near(float x) { return x >= 0.001f; } // (double)x >= 0.001

// interpolator_g<1> (swegl/render/interpolator.hpp:52-104)
struct Interp {
    float top, tstep, alpha, bottom, bstep, v0, dv;

    __device__ __forceinline__ void init_self(float dist, float z1, float z2)
    {
        v0 = z1;
        dv = z2 - z1;
        float alphastep = 1.0f / dist;
        bottom = 1.0f / z1;
        float invz2 = 1.0f / z2;
        alpha = 0.0f;
        top = alpha;
        top = top * bottom;
        tstep = (1.0f * invz2 - top) * alphastep;
        bstep = (invz2 - bottom) * alphastep;
    }
    __device__ __forceinline__ void displace(float move)
    {
        top = top + tstep * move;
        bottom = bottom + bstep * move;
        alpha = top / bottom;
    }
    __device__ __forceinline__ void step()
    {
        top = top + tstep;
        bottom = bottom + bstep;
        alpha = top / bottom;
    }
    __device__ __forceinline__ float value() const { return v0 + dv * alpha; }
};

// line_side (src/render/renderer.cpp:21-26)
struct Side {
    Interp it;
    float ratio;
    float x;
};

// s^p for the specular term.  The reference evaluates pow((double)s, p) and
// rounds it to float (src/render/pixel_shaders.cpp:193).  Here s^p is formed
// by left-to-right binary exponentiation on a pair of floats hi + lo holding
// about 46 bits: a square takes hi * hi, its exact rounding error from one
// fused multiply-add (Dekker's exact product, "A floating-point technique for
// extending the available precision", 1971), and the cross term 2 * hi * lo
// added to that error by one more fused multiply-add (lo * lo, below 2^-46 of
// the value, is dropped); the pair is then renormalised (Dekker's fast two-
// sum).  A multiply by s takes hi * s, its exact error, and lo * s added to
// the error by a fused multiply-add, unnormalised (|lo| stays within a few
// units in the last place of hi).  The pair is rounded to float once at the
// end: the float nearest s^p unless s^p lies within about p * 2^-45 of its
// value from a rounding boundary.  Shininess is 0..1024 (checked at upload).
__host__ __device__ __forceinline__ int top_bit(int p)
{
#ifdef __CUDA_ARCH__
    return 31 - __clz(p);
#else
    return 31 - __builtin_clz((unsigned)p);
#endif
}
__host__ __device__ __forceinline__ float spec_pow(float s, int p)
{
    if (p <= 0)
        return 1.0f;
    float hi = s, lo = 0.0f;
    for (int bit = top_bit(p) - 1; bit >= 0; bit--) {
        const float sq = hi * hi;
        const float err = fmaf(hi, hi, -sq);
        const float low = fmaf(hi + hi, lo, err);
        hi = sq + low;
        lo = low - (hi - sq);
        if ((p >> bit) & 1) {
            const float m = hi * s;
            const float em = fmaf(hi, s, -m);
            lo = fmaf(lo, s, em);
            hi = m;
        }
    }
    return hi + lo;
}

} // namespace sgl
