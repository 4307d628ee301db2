// Single-precision transcendental functions used by the shading code (sincos, exp2, log2, pow,
// atan2, asin), written in plain IEEE arithmetic so that the same source compiled for the device
// (nvcc, -fmad=false) and for the host (g++, -ffp-contract=off) gives identical bits.
//
// Methods (all textbook):
//   sincos : Cody-Waite reduction by pi/2 with a three-term split (1.5703125 + 4.838705e-4 +
//            -4.371139e-8), then Taylor polynomials of sin and cos on [-pi/4, pi/4] (truncation
//            below 1e-11), quadrant selection from the integer multiple.
//   exp2   : x = n + f with |f| <= 1/2, Taylor series of e^(f ln 2) to degree 8, scaled by 2^n.
//   log2   : x = m 2^e with m in [sqrt(1/2), sqrt(2)), ln m = 2 atanh((m-1)/(m+1)) by its series.
//   pow    : exp2(y log2 x) for x > 0, with pow(x, 1) = x, pow(x, 0) = 1, pow(0, y > 0) = 0 and
//            NaN for x < 0, as HLSL's pow.
//   atan2  : reduction to atan on [0, tan(pi/8)] (via atan(a) = pi/4 + atan((a-1)/(a+1))) and its
//            odd Taylor series to degree 19; quadrant fix-up.
//   asin   : atan2(x, sqrt((1 - x)(1 + x))).
// Accuracy (checked against double-precision libm in the tests): a few ulp.
#pragma once

#include <cmath>
#include <cstdint>

#if defined(__CUDACC__)
#define AGB_FM __host__ __device__ __forceinline__
// The larger functions (sincos, exp2, log2, pow, atan2) can be kept out of line on the device so
// that the shading code holds one copy of each instead of one per call site.
#if defined(AGB_FM_OUTLINE)
#define AGB_FMX static __host__ __device__ __noinline__
#else
#define AGB_FMX __host__ __device__ __forceinline__
#endif
#else
#define AGB_FM inline
#define AGB_FMX inline
#endif

namespace agb_fm
{

AGB_FM bool finite_(float x) { return x - x == 0.0f; }
// Sign bit of a non-NaN float (true for -0).
AGB_FM bool negative_(float x) { return x < 0.0f || (x == 0.0f && 1.0f / x < 0.0f); }

AGB_FMX void sincos(float x, float* s, float* c)
{
    if (!finite_(x))
    {
        *s = *c = x - x; // NaN
        return;
    }
    float kf = rintf(x * 0.63661975f);
    if (kf > 1048576.0f || kf < -1048576.0f)
        kf = 0.0f; // outside the reduction's range (never used by the renderer): unreduced
    int k    = int(kf);
    float r  = ((x - kf * 1.5703125f) - kf * 0.00048387050628662109375f) - kf * -4.371139e-08f;
    float r2 = r * r;
    float sp = r + r * r2 * (-1.6666667e-01f + r2 * (8.3333333e-03f + r2 * (-1.9841270e-04f +
                      r2 * (2.7557319e-06f + r2 * -2.5052108e-08f))));
    float cp = 1.0f - 0.5f * r2 + r2 * r2 * (4.1666668e-02f + r2 * (-1.3888889e-03f +
                      r2 * (2.4801587e-05f + r2 * (-2.7557319e-07f + r2 * 2.0876757e-09f))));
    switch (k & 3)
    {
    case 0:
        *s = sp;
        *c = cp;
        break;
    case 1:
        *s = cp;
        *c = -sp;
        break;
    case 2:
        *s = -sp;
        *c = -cp;
        break;
    default:
        *s = -cp;
        *c = sp;
        break;
    }
}

AGB_FMX float exp2(float x)
{
    if (x != x)
        return x;
    if (x >= 128.0f)
        return INFINITY;
    if (x < -150.0f)
        return 0.0f;
    float n = rintf(x);
    float t = (x - n) * 0.6931472f;
    float p = 1.0f + t * (1.0f + t * (0.5f + t * (1.6666667e-01f + t * (4.1666668e-02f +
                      t * (8.3333333e-03f + t * (1.3888889e-03f + t * (1.9841270e-04f +
                      t * 2.4801587e-05f)))))));
    return ldexpf(p, int(n));
}

AGB_FMX float log2(float x)
{
    if (x != x)
        return x;
    if (x < 0.0f)
        return NAN;
    if (x == 0.0f)
        return -INFINITY;
    if (!finite_(x))
        return x;
    int e;
    float m = frexpf(x, &e); // [0.5, 1)
    if (m < 0.70710678f)
    {
        m = m * 2.0f;
        e = e - 1;
    }
    float s  = (m - 1.0f) / (m + 1.0f);
    float s2 = s * s;
    float ln = s * (2.0f + s2 * (6.6666669e-01f + s2 * (4.0000001e-01f + s2 * (2.8571429e-01f +
                   s2 * (2.2222222e-01f + s2 * 1.8181819e-01f)))));
    return float(e) + ln * 1.442695f;
}

AGB_FMX float pow(float x, float y)
{
    if (y == 1.0f)
        return x;
    if (y == 0.0f)
        return 1.0f;
    if (x != x || y != y)
        return x + y;
    if (x < 0.0f)
        return NAN;
    if (x == 0.0f)
        return y > 0.0f ? 0.0f : INFINITY;
    if (x == 1.0f)
        return 1.0f;
    return agb_fm::exp2(y * agb_fm::log2(x));
}

// atan on [0, tan(pi/8)]: odd Taylor series to t^19.
AGB_FM float atanSmall(float t)
{
    float t2 = t * t;
    return t + t * t2 * (-3.3333334e-01f + t2 * (2.0000000e-01f + t2 * (-1.4285715e-01f +
                   t2 * (1.1111111e-01f + t2 * (-9.0909094e-02f + t2 * (7.6923080e-02f +
                   t2 * (-6.6666670e-02f + t2 * (5.8823529e-02f + t2 * -5.2631579e-02f))))))));
}

AGB_FMX float atan2(float y, float x)
{
    if (x != x || y != y)
        return x + y;
    float ax = fabsf(x), ay = fabsf(y);
    if (ax == 0.0f && ay == 0.0f)
        return (x < 0.0f || (x == 0.0f && negative_(x))) ? (negative_(y) ? -3.1415927f : 3.1415927f)
                                                       : (negative_(y) ? -0.0f : 0.0f);
    if (!finite_(ax) || !finite_(ay))
    {
        float q = (!finite_(ax) && !finite_(ay)) ? 0.7853982f : (!finite_(ay) ? 1.5707964f : 0.0f);
        if (x < 0.0f)
            q = 3.1415927f - q;
        return negative_(y) ? -q : q;
    }
    float a = (ay > ax) ? ax / ay : ay / ax;
    float r = a > 0.41421356f ? 0.7853982f + atanSmall((a - 1.0f) / (a + 1.0f)) : atanSmall(a);
    if (ay > ax)
        r = 1.5707964f - r;
    if (x < 0.0f)
        r = 3.1415927f - r;
    return negative_(y) ? -r : r;
}

AGB_FM float asin(float x)
{
    if (x != x || x > 1.0f || x < -1.0f)
        return NAN;
    return agb_fm::atan2(x, sqrtf((1.0f - x) * (1.0f + x)));
}

AGB_FM float sin(float x)
{
    float s, c;
    agb_fm::sincos(x, &s, &c);
    return s;
}
AGB_FM float cos(float x)
{
    float s, c;
    agb_fm::sincos(x, &s, &c);
    return c;
}

} // namespace agb_fm
