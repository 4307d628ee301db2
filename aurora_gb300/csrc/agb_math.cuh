// Device vector math with the HLSL intrinsic semantics Aurora's shaders rely on (lerp, saturate,
// reflect, refract, normalize), kept in the same operation order as the shaders so that FP32
// results track the reference arithmetic (Shaders/Globals.slang, Shaders/Colors.slang).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

// The device build keeps the larger transcendental helpers out of line (one copy each in the
// shading code; measured faster through the instruction cache).
#if defined(__CUDACC__) && !defined(AGB_FM_INLINE)
#define AGB_FM_OUTLINE
#endif
#include "agb_fmath.h"

#define AGB_HD __host__ __device__ __forceinline__
#define AGB_D __device__ __forceinline__
// The large shading functions (BSDF evaluate / sample, environment lookups) are called from
// several places in the shading kernel; keeping one out-of-line copy of each keeps that kernel's
// code within the instruction cache.
#ifdef AGB_BSDF_INLINE
#define AGB_DN __device__ __forceinline__
#else
#define AGB_DN static __device__ __noinline__
#endif

namespace agb
{

struct v2
{
    float x, y;
};
struct v3
{
    float x, y, z;
};

AGB_HD v2 mk2(float a, float b) { return v2{ a, b }; }
AGB_HD v3 mk3(float a, float b, float c) { return v3{ a, b, c }; }
AGB_HD v3 splat(float a) { return v3{ a, a, a }; }
AGB_HD v3 ld3(const float* p) { return v3{ p[0], p[1], p[2] }; }
// Three floats through the read-only data path.
AGB_D v3 ldg3(const float* p) { return v3{ __ldg(p), __ldg(p + 1), __ldg(p + 2) }; }

AGB_HD v3 operator+(v3 a, v3 b) { return v3{ a.x + b.x, a.y + b.y, a.z + b.z }; }
AGB_HD v3 operator-(v3 a, v3 b) { return v3{ a.x - b.x, a.y - b.y, a.z - b.z }; }
AGB_HD v3 operator*(v3 a, v3 b) { return v3{ a.x * b.x, a.y * b.y, a.z * b.z }; }
AGB_HD v3 operator/(v3 a, v3 b) { return v3{ a.x / b.x, a.y / b.y, a.z / b.z }; }
AGB_HD v3 operator*(v3 a, float s) { return v3{ a.x * s, a.y * s, a.z * s }; }
AGB_HD v3 operator*(float s, v3 a) { return v3{ s * a.x, s * a.y, s * a.z }; }
AGB_HD v3 operator/(v3 a, float s) { return v3{ a.x / s, a.y / s, a.z / s }; }
AGB_HD v3 operator-(v3 a) { return v3{ -a.x, -a.y, -a.z }; }
AGB_HD v3& operator+=(v3& a, v3 b)
{
    a = a + b;
    return a;
}
AGB_HD v3& operator*=(v3& a, v3 b)
{
    a = a * b;
    return a;
}
AGB_HD v3& operator*=(v3& a, float s)
{
    a = a * s;
    return a;
}
AGB_HD v3& operator/=(v3& a, float s)
{
    a = a / s;
    return a;
}
AGB_HD v2 operator+(v2 a, v2 b) { return v2{ a.x + b.x, a.y + b.y }; }
AGB_HD v2 operator-(v2 a, v2 b) { return v2{ a.x - b.x, a.y - b.y }; }
AGB_HD v2 operator*(v2 a, float s) { return v2{ a.x * s, a.y * s }; }

AGB_HD float dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
AGB_HD v3 cross(v3 a, v3 b)
{
    return v3{ a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x };
}
AGB_HD float length(v3 a) { return sqrtf(dot(a, a)); }
AGB_HD v3 normalize(v3 a) { return a / sqrtf(dot(a, a)); }
// HLSL lerp(x, y, s) = x + s * (y - x)
AGB_HD float lerpf(float a, float b, float t) { return a + t * (b - a); }
AGB_HD v3 lerp3(v3 a, v3 b, float t) { return a + (b - a) * t; }
AGB_HD v3 lerp3v(v3 a, v3 b, v3 t) { return a + (b - a) * t; }
AGB_HD float clampf(float v, float lo, float hi) { return v < lo ? lo : (v > hi ? hi : v); }
AGB_HD float saturatef(float v) { return clampf(v, 0.f, 1.f); }
AGB_HD v3 clamp3(v3 v, float lo, float hi)
{
    return v3{ clampf(v.x, lo, hi), clampf(v.y, lo, hi), clampf(v.z, lo, hi) };
}
AGB_HD v3 max3(v3 v, float lo)
{
    return v3{ v.x > lo ? v.x : lo, v.y > lo ? v.y : lo, v.z > lo ? v.z : lo };
}
AGB_HD v3 sqrt3(v3 v) { return v3{ sqrtf(v.x), sqrtf(v.y), sqrtf(v.z) }; }
AGB_HD v3 pow3(v3 v, float e) { return v3{ agb_fm::pow(v.x, e), agb_fm::pow(v.y, e), agb_fm::pow(v.z, e) }; }
AGB_HD v3 abs3(v3 v) { return v3{ fabsf(v.x), fabsf(v.y), fabsf(v.z) }; }
AGB_HD bool isBlack(v3 c) { return c.x == 0.f && c.y == 0.f && c.z == 0.f; }
AGB_HD v3 reflect(v3 i, v3 n) { return i - n * (2.f * dot(n, i)); }
AGB_HD v3 refract(v3 i, v3 n, float eta)
{
    float cosi = dot(n, i);
    float k    = 1.f - eta * eta * (1.f - cosi * cosi);
    if (k < 0.f)
        return splat(0.f);
    return i * eta - n * (eta * cosi + sqrtf(k));
}
AGB_HD float sqr(float x) { return x * x; }
AGB_HD float fmaxf_(float a, float b) { return a > b ? a : b; }
AGB_HD float fminf_(float a, float b) { return a < b ? a : b; }

constexpr float kPi      = 3.1415926535897932384626433832795f;
constexpr float kFloatEps = 0.000001f; // M_FLOAT_EPS
constexpr float kRayTMin  = 0.01f;     // M_RAY_TMIN

// Aurora's M_PI_INV macro expands to "1.0 / pi" without parentheses, so "x * M_PI_INV" is a
// division by pi after a multiplication by one.
AGB_HD float divPi(float x) { return (x * 1.0f) / kPi; }
AGB_HD v3 divPi(v3 x) { return (x * 1.0f) / kPi; }

// Colors.slang:26-29
AGB_HD float luminance(v3 v) { return dot(v, v3{ 0.2125f, 0.7154f, 0.0721f }); }

// Lobe and ray-type identifiers (Shaders/BSDFCommon.slang:28-39).
enum : int
{
    TRANSPARENCY_LOBE           = 1,
    COAT_LOBE                   = 2,
    METAL_LOBE                  = 3,
    GLOSSY_LOBE                 = 4,
    TRANSMISSION_LOBE           = 5,
    SHEEN_LOBE                  = 6,
    DIFFUSE_LOBE                = 7,
    NO_SECONDARY_RAY            = 8,
    CAMERA_RAY                  = 9,
    GROUND_PLANE_REFLECTION_RAY = 10
};

// PCG2D (Random.slang:96-137).  The generator's stored state is the last hashed pair.
struct Rng
{
    uint32_t x, y;
};
AGB_HD Rng rngInit(uint32_t sampleIndex, uint32_t screenWidth, uint32_t px, uint32_t py)
{
    return Rng{ py * screenWidth + px, sampleIndex };
}
AGB_HD v2 random2D(Rng& r)
{
    uint32_t vx = r.x, vy = r.y;
    vx += vy * 1664525u;
    vy += vx * 1664525u;
    vx ^= vx >> 16u;
    vy ^= vy >> 16u;
    vx += vy * 1664525u;
    vy += vx * 1664525u;
    vx ^= vx >> 16u;
    vy ^= vy >> 16u;
    r.x = vx;
    r.y = vy;
    // uint -> float rounds to nearest; 0xFFFFFFFF as float is 2^32, an exact power of two.
    return v2{ float(vx) * 2.3283064365386963e-10f, float(vy) * 2.3283064365386963e-10f };
}

// Warp-aggregated append to a queue: one atomicAdd per warp, lanes get consecutive slots.
AGB_D uint32_t warpAppend(uint32_t* counter, bool active)
{
    unsigned mask = __ballot_sync(__activemask(), active);
    if (!active)
        return 0xffffffffu;
    int lane   = threadIdx.x & 31;
    int leader = __ffs(mask) - 1;
    uint32_t base = 0;
    if (lane == leader)
        base = atomicAdd(counter, uint32_t(__popc(mask)));
    base = __shfl_sync(mask, base, leader);
    return base + __popc(mask & ((1u << lane) - 1u));
}

} // namespace agb
