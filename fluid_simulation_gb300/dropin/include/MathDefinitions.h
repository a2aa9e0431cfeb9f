// Drop-in for the reference's include/MathDefinitions.h: the scalar type and
// helpers of the public API, without the Eigen dependency (the GPU library
// replaces Eigen's solver).
#ifndef MATH_DEFINITIONS
#define MATH_DEFINITIONS

#include <math.h>

typedef float MyFloat;  // the reference's default (USE_DOUBLE_PRECISION unset)

// CLAMP(d, min, max) on MyFloat, as include/MathDefinitions.h:16-19.
inline MyFloat CLAMP(MyFloat d, MyFloat min, MyFloat max)
{
    const MyFloat lo = d < min ? min : d;
    return lo > max ? max : lo;
}

inline MyFloat smoothstep(MyFloat edge0, MyFloat edge1, MyFloat x)
{
    const MyFloat t = CLAMP((x - edge0) / (edge1 - edge0), 0, 1);
    return t * t * (3 - 2 * t);
}

inline MyFloat gaussian(MyFloat x, MyFloat sigma, MyFloat mu)
{
    const MyFloat d = x - mu;
    return (1 / (sigma * sqrt(2 * M_PI))) * exp(-(d * d) / (2 * sigma * sigma));
}

#endif
