// A small stand-in for the parts of GLM (OpenGL Mathematics) that Aurora's public header uses:
// float / int vectors of 2-4 components and a 4x4 float matrix, with GLM's memory layout
// (components in order; a matrix is four column vectors, element [c][r] at c * 4 + r) and GLM's
// GLM_FORCE_CTOR_INIT defaults (vectors zero, matrices identity).  Headers that include
// <glm/glm.hpp> compile against it with the same object layout as against GLM itself.
#pragma once

#include <cstddef>

namespace glm
{

template <class T>
struct tvec2
{
    T x, y;
    constexpr tvec2() : x(0), y(0) {}
    constexpr explicit tvec2(T s) : x(s), y(s) {}
    constexpr tvec2(T a, T b) : x(a), y(b) {}
    T& operator[](int i) { return (&x)[i]; }
    const T& operator[](int i) const { return (&x)[i]; }
    bool operator==(const tvec2& o) const { return x == o.x && y == o.y; }
    bool operator!=(const tvec2& o) const { return !(*this == o); }
};

template <class T>
struct tvec3
{
    T x, y, z;
    constexpr tvec3() : x(0), y(0), z(0) {}
    constexpr explicit tvec3(T s) : x(s), y(s), z(s) {}
    constexpr tvec3(T a, T b, T c) : x(a), y(b), z(c) {}
    T& operator[](int i) { return (&x)[i]; }
    const T& operator[](int i) const { return (&x)[i]; }
    bool operator==(const tvec3& o) const { return x == o.x && y == o.y && z == o.z; }
    bool operator!=(const tvec3& o) const { return !(*this == o); }
};

template <class T>
struct tvec4
{
    T x, y, z, w;
    constexpr tvec4() : x(0), y(0), z(0), w(0) {}
    constexpr explicit tvec4(T s) : x(s), y(s), z(s), w(s) {}
    constexpr tvec4(T a, T b, T c, T d) : x(a), y(b), z(c), w(d) {}
    constexpr tvec4(const tvec3<T>& v, T d) : x(v.x), y(v.y), z(v.z), w(d) {}
    T& operator[](int i) { return (&x)[i]; }
    const T& operator[](int i) const { return (&x)[i]; }
    bool operator==(const tvec4& o) const { return x == o.x && y == o.y && z == o.z && w == o.w; }
    bool operator!=(const tvec4& o) const { return !(*this == o); }
};

using vec2  = tvec2<float>;
using vec3  = tvec3<float>;
using vec4  = tvec4<float>;
using ivec2 = tvec2<int>;
using ivec3 = tvec3<int>;
using ivec4 = tvec4<int>;
using uvec2 = tvec2<unsigned int>;

// Column-major 4x4 matrix: m[c] is column c.
struct mat4
{
    vec4 value[4];
    constexpr mat4() : value{ vec4(1, 0, 0, 0), vec4(0, 1, 0, 0), vec4(0, 0, 1, 0), vec4(0, 0, 0, 1) } {}
    constexpr explicit mat4(float s) : value{ vec4(s, 0, 0, 0), vec4(0, s, 0, 0), vec4(0, 0, s, 0), vec4(0, 0, 0, s) }
    {
    }
    constexpr mat4(const vec4& c0, const vec4& c1, const vec4& c2, const vec4& c3) : value{ c0, c1, c2, c3 } {}
    vec4& operator[](int c) { return value[c]; }
    const vec4& operator[](int c) const { return value[c]; }
    bool operator==(const mat4& o) const
    {
        return value[0] == o.value[0] && value[1] == o.value[1] && value[2] == o.value[2] && value[3] == o.value[3];
    }
    bool operator!=(const mat4& o) const { return !(*this == o); }
};

} // namespace glm
