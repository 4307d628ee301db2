// Oracle recipe support (test infrastructure): a stand-in for Aurora's precompiled header, with just
// the names the reference's AliasMap.cpp/.h use (vec1/vec3/uvec2, dot, make_vec3, AU_ASSERT,
// BEGIN_AURORA).  It lets the reference's own AliasMap.cpp compile unmodified, in place, so the oracle's
// restatement of the alias-table build can be checked against the reference itself.
#pragma once

#include <cmath>
#include <cstddef>
#include <cstring>
#include <vector>

#define BEGIN_AURORA                                                                               \
    namespace Aurora                                                                               \
    {
#define END_AURORA }

#define AU_ASSERT(cond, ...)                                                                       \
    do                                                                                             \
    {                                                                                              \
        if (!(cond))                                                                               \
            __builtin_trap();                                                                      \
    } while (0)

namespace shim
{
struct vec3
{
    float x, y, z;
    constexpr vec3(float a, float b, float c) : x(a), y(b), z(c) {}
};
struct uvec2
{
    unsigned int x, y;
};
using vec1 = float;
// glm::dot for vec3 sums in (x, y, z) order.
inline float dot(const vec3& a, const vec3& b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline vec3 make_vec3(const float* p) { return vec3(p[0], p[1], p[2]); }
} // namespace shim

using namespace shim;
using namespace std; // float overloads of sin() as in the reference build
