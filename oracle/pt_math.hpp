// Oracle (test infrastructure, never linked into the product): HLSL-semantics vector math used by
// the CPU restatement of Aurora's path tracer.  Every function is templated on the scalar type so
// the same restatement runs in FP32 (bit-level checks of the CUDA kernels) and FP64 (the accuracy
// reference for converged images).
//
// Follows the intrinsic semantics the reference shaders rely on (Slang/HLSL): lerp, saturate,
// reflect, refract, normalize, sincos, asin, atan2 (Libraries/Aurora/Source/Shaders/*.slang).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>

// The FP32 instantiation uses the product's own transcendental functions (plain IEEE arithmetic,
// identical bits on host and device) so that FP32 parity checks compare the shading algebra and
// not two libm implementations; the FP64 instantiation uses the C++ standard library and is the
// accuracy reference.  agb_fmath.h's accuracy is checked against FP64 libm by the tests.
#include "../aurora_gb300/csrc/agb_fmath.h"

namespace orc
{

inline float tsin(float x) { return agb_fm::sin(x); }
inline float tcos(float x) { return agb_fm::cos(x); }
inline float tpow(float x, float y) { return agb_fm::pow(x, y); }
inline float texp2(float x) { return agb_fm::exp2(x); }
inline float tatan2(float y, float x) { return agb_fm::atan2(y, x); }
inline float tasin(float x) { return agb_fm::asin(x); }
inline double tsin(double x) { return std::sin(x); }
inline double tcos(double x) { return std::cos(x); }
inline double tpow(double x, double y) { return std::pow(x, y); }
inline double texp2(double x) { return std::exp2(x); }
inline double tatan2(double y, double x) { return std::atan2(y, x); }
inline double tasin(double x) { return std::asin(x); }

template <class T>
struct V2
{
    T x = 0, y = 0;
    V2() = default;
    V2(T a, T b) : x(a), y(b) {}
    explicit V2(T a) : x(a), y(a) {}
    V2 operator+(const V2& o) const { return V2(x + o.x, y + o.y); }
    V2 operator-(const V2& o) const { return V2(x - o.x, y - o.y); }
    V2 operator*(const V2& o) const { return V2(x * o.x, y * o.y); }
    V2 operator/(const V2& o) const { return V2(x / o.x, y / o.y); }
    V2 operator*(T s) const { return V2(x * s, y * s); }
    V2 operator/(T s) const { return V2(x / s, y / s); }
    T& operator[](int i) { return i == 0 ? x : y; }
    T operator[](int i) const { return i == 0 ? x : y; }
};

template <class T>
struct V3
{
    T x = 0, y = 0, z = 0;
    V3() = default;
    V3(T a, T b, T c) : x(a), y(b), z(c) {}
    explicit V3(T a) : x(a), y(a), z(a) {}
    template <class U>
    static V3 from(const U* p)
    {
        return V3(T(p[0]), T(p[1]), T(p[2]));
    }
    V3 operator+(const V3& o) const { return V3(x + o.x, y + o.y, z + o.z); }
    V3 operator-(const V3& o) const { return V3(x - o.x, y - o.y, z - o.z); }
    V3 operator*(const V3& o) const { return V3(x * o.x, y * o.y, z * o.z); }
    V3 operator/(const V3& o) const { return V3(x / o.x, y / o.y, z / o.z); }
    V3 operator*(T s) const { return V3(x * s, y * s, z * s); }
    V3 operator/(T s) const { return V3(x / s, y / s, z / s); }
    V3 operator-() const { return V3(-x, -y, -z); }
    V3& operator+=(const V3& o)
    {
        x += o.x;
        y += o.y;
        z += o.z;
        return *this;
    }
    V3& operator*=(const V3& o)
    {
        x *= o.x;
        y *= o.y;
        z *= o.z;
        return *this;
    }
    V3& operator*=(T s)
    {
        x *= s;
        y *= s;
        z *= s;
        return *this;
    }
    V3& operator/=(T s)
    {
        x /= s;
        y /= s;
        z /= s;
        return *this;
    }
    V3& operator/=(const V3& o)
    {
        x /= o.x;
        y /= o.y;
        z /= o.z;
        return *this;
    }
    T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    T operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
};

template <class T>
inline V3<T> operator*(T s, const V3<T>& v)
{
    return V3<T>(s * v.x, s * v.y, s * v.z);
}
template <class T>
inline V2<T> operator*(T s, const V2<T>& v)
{
    return V2<T>(s * v.x, s * v.y);
}

template <class T>
inline T dot(const V3<T>& a, const V3<T>& b)
{
    return a.x * b.x + a.y * b.y + a.z * b.z;
}
template <class T>
inline V3<T> cross(const V3<T>& a, const V3<T>& b)
{
    return V3<T>(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
template <class T>
inline T length(const V3<T>& a)
{
    return std::sqrt(dot(a, a));
}
template <class T>
inline V3<T> normalize(const V3<T>& a)
{
    return a / std::sqrt(dot(a, a));
}
// HLSL lerp(x, y, s) = x + s * (y - x).
template <class T>
inline T lerp(T a, T b, T t)
{
    return a + t * (b - a);
}
template <class T>
inline V3<T> lerp(const V3<T>& a, const V3<T>& b, T t)
{
    return a + (b - a) * t;
}
template <class T>
inline T clampT(T v, T lo, T hi)
{
    return v < lo ? lo : (v > hi ? hi : v);
}
template <class T>
inline T saturate(T v)
{
    return clampT(v, T(0), T(1));
}
template <class T>
inline V3<T> clamp3(const V3<T>& v, T lo, T hi)
{
    return V3<T>(clampT(v.x, lo, hi), clampT(v.y, lo, hi), clampT(v.z, lo, hi));
}
template <class T>
inline V3<T> max3(const V3<T>& v, T lo)
{
    return V3<T>(v.x > lo ? v.x : lo, v.y > lo ? v.y : lo, v.z > lo ? v.z : lo);
}
template <class T>
inline V3<T> sqrt3(const V3<T>& v)
{
    return V3<T>(std::sqrt(v.x), std::sqrt(v.y), std::sqrt(v.z));
}
template <class T>
inline V3<T> pow3(const V3<T>& v, T e)
{
    return V3<T>(tpow(v.x, e), tpow(v.y, e), tpow(v.z, e));
}
template <class T>
inline V3<T> abs3(const V3<T>& v)
{
    return V3<T>(std::fabs(v.x), std::fabs(v.y), std::fabs(v.z));
}
template <class T>
inline bool isBlack(const V3<T>& c)
{
    return c.x == T(0) && c.y == T(0) && c.z == T(0);
}
// HLSL reflect(i, n) = i - 2 * dot(n, i) * n.
template <class T>
inline V3<T> reflect(const V3<T>& i, const V3<T>& n)
{
    return i - n * (T(2) * dot(n, i));
}
// HLSL refract(i, n, eta): zero vector on total internal reflection.
template <class T>
inline V3<T> refract(const V3<T>& i, const V3<T>& n, T eta)
{
    T cosi = dot(n, i);
    T k    = T(1) - eta * eta * (T(1) - cosi * cosi);
    if (k < T(0))
        return V3<T>(T(0));
    return i * eta - n * (eta * cosi + std::sqrt(k));
}

template <class T>
struct Consts
{
    static constexpr T PI     = T(3.1415926535897932384626433832795);
    static constexpr T PI_INV = T(1.0 / 3.1415926535897932384626433832795);
    // M_FLOAT_EPS and M_RAY_TMIN (Shaders/Globals.slang:26,29; StandardSurfaceBSDF.slang).
    static constexpr T FLOAT_EPS = T(0.000001f);
    static constexpr T RAY_TMIN  = T(0.01f);
};

// Perceived luminance (Shaders/Colors.slang:26-29).
template <class T>
inline T luminance(const V3<T>& v)
{
    return dot(v, V3<T>(T(0.2125f), T(0.7154f), T(0.0721f)));
}

// Fast sRGB approximation (Shaders/Colors.slang:33-40).
template <class T>
inline V3<T> linearTosRGB(const V3<T>& c)
{
    V3<T> s1 = sqrt3(c);
    V3<T> s2 = sqrt3(s1);
    V3<T> s3 = sqrt3(s2);
    return s1 * T(0.662002687f) + s2 * T(0.684122060f) - s3 * T(0.323583601f) -
        c * T(0.0225411470f);
}

// ACES filmic curve (Shaders/Colors.slang:44-53).
template <class T>
inline V3<T> toneMapACES(const V3<T>& c)
{
    const T a = T(2.51f), b = T(0.03f), cc = T(2.43f), d = T(0.59f), e = T(0.14f);
    V3<T> num = c * (c * a + V3<T>(b));
    V3<T> den = c * (c * cc + V3<T>(d)) + V3<T>(e);
    return clamp3(num / den, T(0), T(1));
}

// 3x4 row-major affine transform (rows of a float3x4): p' = M * (p, 1).
template <class T>
struct Xform
{
    T m[12];
    V3<T> point(const V3<T>& p) const
    {
        return V3<T>(m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3],
            m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7],
            m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11]);
    }
    V3<T> vector(const V3<T>& v) const
    {
        return V3<T>(m[0] * v.x + m[1] * v.y + m[2] * v.z, m[4] * v.x + m[5] * v.y + m[6] * v.z,
            m[8] * v.x + m[9] * v.y + m[10] * v.z);
    }
};

} // namespace orc
