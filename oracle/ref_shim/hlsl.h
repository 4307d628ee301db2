// HLSL / Slang vocabulary for compiling the reference's shader sources as host C++ (test
// infrastructure: the oracle's pin, never part of the product).
//
// oracle/build_oracle.py rewrites the reference's .slang files mechanically (out / inout
// parameters to references, scalar swizzles to constructors, vector swizzles to accessor calls,
// unsuffixed floating literals to float literals, as HLSL types them) into oracle/_ref/gen/, and
// compiles them against this header.  The semantics restated here follow the HLSL intrinsic
// reference: lerp(a, b, s) = a + s (b - a), saturate = clamp to [0, 1], refract / reflect as
// defined there, component-wise vector arithmetic, scalars splatting to vectors.  Transcendentals
// call the C library in the scalar's precision.
//
// REF_REAL selects the scalar type of the float vectors: float for the FP32 pin, double for the
// FP64 one (where the generated code's `float` is redefined to double by the including file).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <type_traits>

// The C library's M_PI is a double constant; the shaders define their own float one when M_PI is
// not yet defined (Globals.slang), which is the one they are compiled with.
#undef M_PI

#ifndef REF_REAL
#define REF_REAL float
#endif

namespace hlsl
{

typedef REF_REAL real;

template <class T, int N>
struct Vec;

template <class T>
struct Vec<T, 2>
{
    T x, y;
    Vec() : x(0), y(0) {}
    Vec(T s) : x(s), y(s) {}
    Vec(T a, T b) : x(a), y(b) {}
    template <class U>
    explicit Vec(const Vec<U, 2>& o) : x(T(o.x)), y(T(o.y))
    {
    }
    T& operator[](int i) { return i == 0 ? x : y; }
    T operator[](int i) const { return i == 0 ? x : y; }
};

template <class T>
struct Vec<T, 3>
{
    T x, y, z;
    Vec() : x(0), y(0), z(0) {}
    Vec(T s) : x(s), y(s), z(s) {}
    Vec(T a, T b, T c) : x(a), y(b), z(c) {}
    Vec(const Vec<T, 2>& v, T c) : x(v.x), y(v.y), z(c) {}
    template <class U>
    explicit Vec(const Vec<U, 3>& o) : x(T(o.x)), y(T(o.y)), z(T(o.z))
    {
    }
    T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
    T operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
    Vec<T, 2> xy() const { return Vec<T, 2>(x, y); }
};

template <class T>
struct Vec<T, 4>
{
    T x, y, z, w;
    Vec() : x(0), y(0), z(0), w(0) {}
    Vec(T s) : x(s), y(s), z(s), w(s) {}
    Vec(T a, T b, T c, T d) : x(a), y(b), z(c), w(d) {}
    Vec(const Vec<T, 3>& v, T d) : x(v.x), y(v.y), z(v.z), w(d) {}
    Vec(const Vec<T, 2>& a, const Vec<T, 2>& b) : x(a.x), y(a.y), z(b.x), w(b.y) {}
    T& operator[](int i) { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
    T operator[](int i) const { return i == 0 ? x : (i == 1 ? y : (i == 2 ? z : w)); }
    Vec<T, 3> xyz() const { return Vec<T, 3>(x, y, z); }
    Vec<T, 3> rgb() const { return Vec<T, 3>(x, y, z); }
    Vec<T, 2> xy() const { return Vec<T, 2>(x, y); }
    Vec<T, 2> zw() const { return Vec<T, 2>(z, w); }
};

// Component-wise arithmetic, with a scalar on either side splatting.
#define HLSL_BINOP(op)                                                                            \
    template <class T, int N>                                                                     \
    Vec<T, N> operator op(const Vec<T, N>& a, const Vec<T, N>& b)                                 \
    {                                                                                             \
        Vec<T, N> r;                                                                              \
        for (int i = 0; i < N; i++)                                                               \
            r[i] = a[i] op b[i];                                                                  \
        return r;                                                                                 \
    }                                                                                             \
    template <class T, int N, class S>                                                            \
    Vec<T, N> operator op(const Vec<T, N>& a, S b)                                                \
    {                                                                                             \
        return a op Vec<T, N>(T(b));                                                              \
    }                                                                                             \
    template <class T, int N, class S>                                                            \
    Vec<T, N> operator op(S a, const Vec<T, N>& b)                                                \
    {                                                                                             \
        return Vec<T, N>(T(a)) op b;                                                              \
    }
HLSL_BINOP(+)
HLSL_BINOP(-)
HLSL_BINOP(*)
HLSL_BINOP(/)
HLSL_BINOP(^)
HLSL_BINOP(>>)
HLSL_BINOP(<<)
HLSL_BINOP(&)
HLSL_BINOP(|)
#undef HLSL_BINOP

// An unsigned vector divided by a floating scalar converts to a floating vector first.
template <int N>
Vec<real, N> operator/(const Vec<uint32_t, N>& a, float b)
{
    Vec<real, N> r;
    for (int i = 0; i < N; i++)
        r[i] = real(a[i]) / real(b);
    return r;
}
template <int N>
Vec<real, N> operator/(const Vec<uint32_t, N>& a, double b)
{
    Vec<real, N> r;
    for (int i = 0; i < N; i++)
        r[i] = real(a[i]) / real(b);
    return r;
}

template <class T, int N>
Vec<T, N> operator-(const Vec<T, N>& a)
{
    Vec<T, N> r;
    for (int i = 0; i < N; i++)
        r[i] = -a[i];
    return r;
}

#define HLSL_ASSIGN(op, bop)                                                                      \
    template <class T, int N, class S>                                                            \
    Vec<T, N>& operator op(Vec<T, N>& a, const S& b)                                              \
    {                                                                                             \
        a = a bop b;                                                                              \
        return a;                                                                                 \
    }
HLSL_ASSIGN(+=, +)
HLSL_ASSIGN(-=, -)
HLSL_ASSIGN(*=, *)
HLSL_ASSIGN(/=, /)
#undef HLSL_ASSIGN

// Comparisons yield boolean vectors.
template <int N>
struct BoolVec
{
    bool v[N];
};
#define HLSL_CMP(op)                                                                              \
    template <class T, int N>                                                                     \
    BoolVec<N> operator op(const Vec<T, N>& a, const Vec<T, N>& b)                                \
    {                                                                                             \
        BoolVec<N> r;                                                                             \
        for (int i = 0; i < N; i++)                                                               \
            r.v[i] = a[i] op b[i];                                                                \
        return r;                                                                                 \
    }                                                                                             \
    template <class T, int N, class S>                                                            \
    BoolVec<N> operator op(const Vec<T, N>& a, S b)                                               \
    {                                                                                             \
        return a op Vec<T, N>(T(b));                                                              \
    }
HLSL_CMP(==)
HLSL_CMP(!=)
HLSL_CMP(<)
HLSL_CMP(>)
HLSL_CMP(<=)
HLSL_CMP(>=)
#undef HLSL_CMP

template <int N>
bool all(const BoolVec<N>& b)
{
    for (int i = 0; i < N; i++)
        if (!b.v[i])
            return false;
    return true;
}
template <int N>
bool any(const BoolVec<N>& b)
{
    for (int i = 0; i < N; i++)
        if (b.v[i])
            return true;
    return false;
}

// Scalar intrinsics in the scalar's own precision.  The generated shader code is compiled inside
// this namespace, so these overloads hide the C library's global ones.
inline float sqrt(float x) { return std::sqrt(x); }
inline double sqrt(double x) { return std::sqrt(x); }
inline float pow(float x, float y) { return std::pow(x, y); }
inline double pow(double x, double y) { return std::pow(x, y); }
inline double pow(double x, float y) { return std::pow(x, double(y)); }
inline double pow(float x, double y) { return std::pow(double(x), y); }
#define HLSL_UNARY(fn)                                                                            \
    inline float fn(float x) { return std::fn(x); }                                               \
    inline double fn(double x) { return std::fn(x); }                                             \
    template <class T, int N>                                                                     \
    Vec<T, N> fn(const Vec<T, N>& a)                                                              \
    {                                                                                             \
        Vec<T, N> r;                                                                              \
        for (int i = 0; i < N; i++)                                                               \
            r[i] = fn(a[i]);                                                                      \
        return r;                                                                                 \
    }
HLSL_UNARY(sin)
HLSL_UNARY(cos)
HLSL_UNARY(tan)
HLSL_UNARY(asin)
HLSL_UNARY(acos)
HLSL_UNARY(atan)
HLSL_UNARY(exp)
HLSL_UNARY(exp2)
HLSL_UNARY(log)
HLSL_UNARY(log2)
HLSL_UNARY(floor)
HLSL_UNARY(ceil)
#undef HLSL_UNARY
inline float abs(float x) { return std::fabs(x); }
inline double abs(double x) { return std::fabs(x); }
inline int abs(int x) { return x < 0 ? -x : x; }
template <class T, int N>
Vec<T, N> abs(const Vec<T, N>& a)
{
    Vec<T, N> r;
    for (int i = 0; i < N; i++)
        r[i] = abs(a[i]);
    return r;
}
template <class T, int N>
Vec<T, N> sqrt(const Vec<T, N>& a)
{
    Vec<T, N> r;
    for (int i = 0; i < N; i++)
        r[i] = sqrt(a[i]);
    return r;
}
template <class T, int N, class S>
Vec<T, N> pow(const Vec<T, N>& a, const S& b)
{
    Vec<T, N> e(b), r;
    for (int i = 0; i < N; i++)
        r[i] = pow(a[i], e[i]);
    return r;
}
inline float atan2(float y, float x) { return std::atan2(y, x); }
inline double atan2(double y, double x) { return std::atan2(y, x); }
inline void sincos(float x, float& s, float& c)
{
    s = std::sin(x);
    c = std::cos(x);
}
inline void sincos(double x, double& s, double& c)
{
    s = std::sin(x);
    c = std::cos(x);
}
inline float radians(float x) { return x * (3.1415926535897932384626433832795f / 180.0f); }
inline double radians(double x) { return x * (3.1415926535897932384626433832795 / 180.0); }

// min / max / clamp / saturate / lerp: scalars, vectors and scalar-vector mixes.  HLSL min and max
// return the other operand when one is NaN; these keep fmin / fmax's choice.
inline float min(float a, float b) { return std::fmin(a, b); }
inline double min(double a, double b) { return std::fmin(a, b); }
inline float max(float a, float b) { return std::fmax(a, b); }
inline double max(double a, double b) { return std::fmax(a, b); }
inline double min(double a, float b) { return std::fmin(a, double(b)); }
inline double min(float a, double b) { return std::fmin(double(a), b); }
inline double max(double a, float b) { return std::fmax(a, double(b)); }
inline double max(float a, double b) { return std::fmax(double(a), b); }
inline int min(int a, int b) { return a < b ? a : b; }
inline int max(int a, int b) { return a > b ? a : b; }
inline uint32_t min(uint32_t a, uint32_t b) { return a < b ? a : b; }
inline uint32_t max(uint32_t a, uint32_t b) { return a > b ? a : b; }
template <class T, int N, class S>
Vec<T, N> min(const Vec<T, N>& a, const S& b)
{
    Vec<T, N> c(b), r;
    for (int i = 0; i < N; i++)
        r[i] = min(a[i], c[i]);
    return r;
}
template <class T, int N, class S>
Vec<T, N> max(const Vec<T, N>& a, const S& b)
{
    Vec<T, N> c(b), r;
    for (int i = 0; i < N; i++)
        r[i] = max(a[i], c[i]);
    return r;
}
template <class T, int N>
Vec<T, N> max(T a, const Vec<T, N>& b)
{
    return max(b, a);
}
template <class T, int N>
Vec<T, N> min(T a, const Vec<T, N>& b)
{
    return min(b, a);
}
// Scalar clamp in the type of the clamped value (bounds convert to it).
template <class A, class B, class C, typename std::enable_if<std::is_arithmetic<A>::value, int>::type = 0>
A clamp(A x, B lo, C hi)
{
    return min(max(x, A(lo)), A(hi));
}
template <class T, int N, class S1, class S2>
Vec<T, N> clamp(const Vec<T, N>& x, const S1& lo, const S2& hi)
{
    return min(max(x, Vec<T, N>(lo)), Vec<T, N>(hi));
}
inline float saturate(float x) { return clamp(x, 0.0f, 1.0f); }
inline double saturate(double x) { return clamp(x, 0.0, 1.0); }
template <class T, int N>
Vec<T, N> saturate(const Vec<T, N>& x)
{
    return clamp(x, T(0), T(1));
}
inline float lerp(float a, float b, float s) { return a + s * (b - a); }
inline double lerp(double a, double b, double s) { return a + s * (b - a); }
template <class T, int N, class S>
Vec<T, N> lerp(const Vec<T, N>& a, const Vec<T, N>& b, const S& s)
{
    return a + Vec<T, N>(s) * (b - a);
}
template <class T, int N, class B, class S, typename std::enable_if<std::is_arithmetic<B>::value, int>::type = 0>
Vec<T, N> lerp(const Vec<T, N>& a, B b, const S& s)
{
    return lerp(a, Vec<T, N>(T(b)), s);
}
template <class T, int N, class A, class S, typename std::enable_if<std::is_arithmetic<A>::value, int>::type = 0>
Vec<T, N> lerp(A a, const Vec<T, N>& b, const S& s)
{
    return lerp(Vec<T, N>(T(a)), b, s);
}

// Geometry.
template <class T, int N>
T dot(const Vec<T, N>& a, const Vec<T, N>& b)
{
    T s = a[0] * b[0];
    for (int i = 1; i < N; i++)
        s = s + a[i] * b[i];
    return s;
}
template <class T>
Vec<T, 3> cross(const Vec<T, 3>& a, const Vec<T, 3>& b)
{
    return Vec<T, 3>(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
template <class T, int N>
T length(const Vec<T, N>& a)
{
    return sqrt(dot(a, a));
}
template <class T, int N>
Vec<T, N> normalize(const Vec<T, N>& a)
{
    return a / length(a);
}
template <class T>
Vec<T, 3> reflect(const Vec<T, 3>& i, const Vec<T, 3>& n)
{
    return i - T(2) * dot(n, i) * n;
}
template <class T, class S>
Vec<T, 3> refract(const Vec<T, 3>& i, const Vec<T, 3>& n, S etaIn)
{
    T eta  = T(etaIn);
    T cosi = dot(n, i);
    T k    = T(1) - eta * eta * (T(1) - cosi * cosi);
    if (k < T(0))
        return Vec<T, 3>(T(0));
    return eta * i - (eta * cosi + sqrt(k)) * n;
}

// Row-major 4x4 matrix (the 16-scalar constructor fills row by row); mul(m, v) treats v as a
// column.
template <class T>
struct Mat4
{
    Vec<T, 4> row[4];
    Mat4() {}
    template <class... S>
    Mat4(S... s)
    {
        static_assert(sizeof...(S) == 16, "float4x4 takes 16 scalars");
        const T v[16] = { T(s)... };
        for (int r = 0; r < 4; r++)
            row[r] = Vec<T, 4>(v[4 * r], v[4 * r + 1], v[4 * r + 2], v[4 * r + 3]);
    }
    Vec<T, 4>& operator[](int i) { return row[i]; }
    const Vec<T, 4>& operator[](int i) const { return row[i]; }
};
template <class T>
Vec<T, 4> mul(const Mat4<T>& m, const Vec<T, 4>& v)
{
    return Vec<T, 4>(dot(m[0], v), dot(m[1], v), dot(m[2], v), dot(m[3], v));
}

// Resources (host stand-ins): a texture of float4 texels, rows from the top, and a sampler whose
// filter is nearest or bilinear with repeat addressing.
struct SamplerState
{
    int linear = 0;
};
template <class Texel>
struct Texture2D
{
    const float* rgba = nullptr; // width * height * 4 floats
    uint32_t width = 0, height = 0;
    void GetDimensions(uint32_t& w, uint32_t& h) const
    {
        w = width;
        h = height;
    }
    Vec<real, 4> texel(int x, int y) const
    {
        const float* p = rgba + (size_t(y) * width + x) * 4;
        return Vec<real, 4>(real(p[0]), real(p[1]), real(p[2]), real(p[3]));
    }
    template <class I3>
    Vec<real, 4> Load(const I3& xy) const
    {
        return texel(int(xy.x), int(xy.y));
    }
    static int wrap(int i, int n)
    {
        int r = i % n;
        return r < 0 ? r + n : r;
    }
    // Texel centres at (i + 0.5) / size; nearest picks the texel containing uv, bilinear blends the
    // four surrounding centres; both wrap.
    Vec<real, 4> SampleLevel(const SamplerState& s, const Vec<real, 2>& uv, real) const
    {
        real fx = uv.x * real(width), fy = uv.y * real(height);
        if (!s.linear)
            return texel(wrap(int(std::floor(fx)), int(width)), wrap(int(std::floor(fy)), int(height)));
        real px = fx - real(0.5), py = fy - real(0.5);
        real x0f = std::floor(px), y0f = std::floor(py);
        real ax = px - x0f, ay = py - y0f;
        int x0 = wrap(int(x0f), int(width)), y0 = wrap(int(y0f), int(height));
        int x1 = wrap(int(x0f) + 1, int(width)), y1 = wrap(int(y0f) + 1, int(height));
        Vec<real, 4> a = lerp(texel(x0, y0), texel(x1, y0), ax);
        Vec<real, 4> b = lerp(texel(x0, y1), texel(x1, y1), ax);
        return lerp(a, b, ay);
    }
};
template <class E>
struct StructuredBuffer
{
    const E* data = nullptr;
    const E& operator[](uint32_t i) const { return data[i]; }
};

} // namespace hlsl

typedef uint32_t uint;
typedef hlsl::Vec<hlsl::real, 2> float2;
typedef hlsl::Vec<hlsl::real, 3> float3;
typedef hlsl::Vec<hlsl::real, 4> float4;
typedef hlsl::Mat4<hlsl::real> float4x4;
typedef hlsl::Vec<int, 2> int2;
typedef hlsl::Vec<int, 3> int3;
typedef hlsl::Vec<uint32_t, 2> uint2;
typedef hlsl::Vec<uint32_t, 3> uint3;
using hlsl::SamplerState;
using hlsl::StructuredBuffer;
using hlsl::Texture2D;
using namespace hlsl;
