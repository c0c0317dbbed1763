/* Portable replacement for the two SSE names swegl uses (__m128 and
 * _mm_add_ps in src/render/colors.cpp); lane-wise IEEE float adds, the same
 * bits as the SSE instruction.  Only used where <xmmintrin.h> is absent. */
#pragma once
#include <stdlib.h>
typedef float __m128 __attribute__((vector_size(16)));
static inline __m128 _mm_add_ps(__m128 a, __m128 b) { return a + b; }
