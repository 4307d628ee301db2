// Autodesk Standard Surface BSDF on the device: evaluation, one-lobe sampling and
// evaluation-with-pdf, matching Aurora's shader semantics
// (Shaders/StandardSurfaceBSDF.slang:22-1372, Shaders/BSDFCommon.slang:76-299,
// Shaders/Sampling.slang:20-107) with the non-denoising lobe selection
// (getGlossySelectionProbability = specLuminance, StandardSurfaceBSDF.slang:193-235).
// Arithmetic follows the shader's operation order so FP32 results agree with it to rounding.
#pragma once

#include "../../include/agb.h"
#include "agb_math.cuh"
#include "agb_sheen_lut.cuh"

// Lobe-level functions: out of line by default so that the three Standard Surface entry points
// share one copy of each (the shading kernel's speed follows its instruction-cache footprint).
#if defined(AGB_LOBE_INLINE)
#define AGB_DL __device__ __forceinline__
#else
#define AGB_DL static __device__ __noinline__
#endif

namespace agb
{

// Material values used during shading (Shaders/Material.slang:20-57).  The values a texture or
// an option can change per hit are held here; the rest are read through `b` from the material
// block, which every lane shading that material shares in L1 (a per-lane copy of all of them
// would sit in each thread's local memory).
struct Mat
{
    const agb_material* b;
    v3 baseColor;
    float specularRoughness;
    float coatRoughness;
    v3 emissionColor;
    v3 opacity;
    AGB_D float base() const { return __ldg(&b->base); }
    AGB_D float diffuseRoughness() const { return __ldg(&b->diffuse_roughness); }
    AGB_D float metalness() const { return __ldg(&b->metalness); }
    AGB_D float specular() const { return __ldg(&b->specular); }
    AGB_D float specularIOR() const { return __ldg(&b->specular_IOR); }
    AGB_D float specularAnisotropy() const { return __ldg(&b->specular_anisotropy); }
    AGB_D float specularRotation() const { return __ldg(&b->specular_rotation); }
    AGB_D float transmission() const { return __ldg(&b->transmission); }
    AGB_D float subsurface() const { return __ldg(&b->subsurface); }
    AGB_D float sheen() const { return __ldg(&b->sheen); }
    AGB_D float sheenRoughness() const { return __ldg(&b->sheen_roughness); }
    AGB_D float coat() const { return __ldg(&b->coat); }
    AGB_D float coatAnisotropy() const { return __ldg(&b->coat_anisotropy); }
    AGB_D float coatRotation() const { return __ldg(&b->coat_rotation); }
    AGB_D float coatIOR() const { return __ldg(&b->coat_IOR); }
    AGB_D float coatAffectColor() const { return __ldg(&b->coat_affect_color); }
    AGB_D float coatAffectRoughness() const { return __ldg(&b->coat_affect_roughness); }
    AGB_D float emission() const { return __ldg(&b->emission); }
    AGB_D v3 specularColor() const { return ldg3(b->specular_color); }
    AGB_D v3 transmissionColor() const { return ldg3(b->transmission_color); }
    AGB_D v3 subsurfaceColor() const { return ldg3(b->subsurface_color); }
    AGB_D v3 sheenColor() const { return ldg3(b->sheen_color); }
    AGB_D v3 coatColor() const { return ldg3(b->coat_color); }
    AGB_D bool thinWalled() const { return __ldg(&b->thin_walled) != 0; }
    AGB_D v3 metalColor() const { return baseColor; } // DefaultMaterial.slang:236
};

// Shading frame.
struct Frame
{
    v3 N, X, Y; // normal, tangent, bitangent
};

// ------------------------------------------------------------------------------------- Sampling
AGB_D v3 sampleUniformDirection(v2 r, float& pdf)
{
    float cosTheta = 1.f - 2.f * r.y;
    float sinTheta = sqrtf(1.f - cosTheta * cosTheta);
    float phi      = 2.f * kPi * r.x;
    float s, c;
    agb_fm::sincos(phi, &s, &c);
    pdf = divPi(0.25f);
    return v3{ sinTheta * c, sinTheta * s, cosTheta };
}
AGB_D v3 sampleHemisphereAbout(v2 r, v3 normal, float& pdf)
{
    v3 d = sampleUniformDirection(r, pdf);
    d    = normalize(normal + d);
    pdf  = divPi(dot(normal, d));
    return d;
}
AGB_D void buildBasis(v3 n, v3& t, v3& b)
{
    b = fabsf(n.y) < 0.999f ? v3{ 0.f, 1.f, 0.f } : v3{ 1.f, 0.f, 0.f };
    t = normalize(cross(b, n));
    b = cross(n, t);
}
AGB_D v3 sampleCone(v2 r, v3 dir, float cosThetaMax)
{
    v3 xb, yb;
    buildBasis(dir, xb, yb);
    float cosTheta = (1.f - r.x) + r.x * cosThetaMax;
    float sinTheta = sqrtf(1.f - cosTheta * cosTheta);
    float phi      = r.y * 2.f * kPi;
    float s, c;
    agb_fm::sincos(phi, &s, &c);
    return xb * c * sinTheta + yb * s * sinTheta + dir * cosTheta;
}
AGB_D v2 sampleDisk(v2 r, float radius)
{
    float rr  = radius * sqrtf(r.x);
    float phi = 2.f * kPi * r.y;
    float s, c;
    agb_fm::sincos(phi, &s, &c);
    return v2{ c * rr, s * rr };
}
AGB_D float misWeight(float f, float g) { return (f * f) / (f * f + g * g); }

// ------------------------------------------------------------------------------- GGX helpers
AGB_D v3 toTangent(v3 i, const Frame& f) { return v3{ dot(i, f.X), dot(i, f.Y), dot(i, f.N) }; }
AGB_D v3 toWorld(v3 i, const Frame& f) { return f.X * i.x + f.Y * i.y + f.N * i.z; }

AGB_D float ggxLambda(v3 v, v2 a)
{
    float squared = (sqr(a.x) * sqr(v.x) + sqr(a.y) * sqr(v.y)) / sqr(v.z);
    return (-1.f + sqrtf(1.f + squared)) * 0.5f;
}
AGB_D float ggxNDF(v3 H, v2 a)
{
    float ellipse = sqr(H.x) / sqr(a.x) + sqr(H.y) / sqr(a.y) + sqr(H.z);
    return 1.f / (kPi * a.x * a.y * sqr(ellipse));
}
AGB_D float ggxVNDF(v3 V, v3 H, v2 a)
{
    float VdotH = dot(V, H);
    if (VdotH <= 0.f)
        return 0.f;
    float D  = ggxNDF(H, a);
    float G1 = dot(V, H) <= 0.f ? 0.f : 1.f / (1.f + ggxLambda(V, a));
    return D * G1 * VdotH / fabsf(V.z);
}
AGB_DL v3 sampleGGXVNDF(v3 V, v2 a, v2 r)
{
    v3 Vh     = normalize(v3{ a.x * V.x, a.y * V.y, V.z });
    float lsq = Vh.x * Vh.x + Vh.y * Vh.y;
    v3 T1     = lsq > 0.f ? v3{ -Vh.y, Vh.x, 0.f } / sqrtf(lsq) : v3{ 1.f, 0.f, 0.f };
    v3 T2     = cross(Vh, T1);
    float rr  = sqrtf(r.x);
    float phi = 2.f * kPi * r.y;
    float s, c;
    agb_fm::sincos(phi, &s, &c);
    float t1 = rr * c;
    float t2 = rr * s;
    float sv = 0.5f * (1.f + Vh.z);
    t2       = (1.f - sv) * sqrtf(1.f - t1 * t1) + sv * t2;
    v3 Nh    = T1 * t1 + T2 * t2 + Vh * sqrtf(fmaxf_(0.f, 1.f - t1 * t1 - t2 * t2));
    return normalize(v3{ a.x * Nh.x, a.y * Nh.y, fmaxf_(0.f, Nh.z) });
}

// ------------------------------------------------------------------------- MaterialX lobes
AGB_D bool sameHemi(v3 a, v3 b, v3 n) { return dot(a, n) * dot(b, n) > 0.f; }
AGB_D v2 roughnessAniso(float roughness, float anisotropy)
{
    float rsq = clampf(roughness * roughness, kFloatEps, 1.f);
    if (anisotropy > 0.f)
    {
        float aspect = sqrtf(1.f - clampf(anisotropy, 0.f, 0.98f));
        return v2{ fminf_(rsq / aspect, 1.f), rsq * aspect };
    }
    return v2{ rsq, rsq };
}
AGB_D float pow5(float x) { return sqr(sqr(x)) * x; }
AGB_D v3 mxMix(v3 bg, v3 fg, float w) { return lerp3(bg, fg, clampf(w, 0.f, 1.f)); }
AGB_DL float orenNayar(v3 L, v3 V, v3 N, float NdotL, float roughness)
{
    float LdotV  = dot(L, V);
    float NdotV  = fabsf(dot(N, V));
    float t      = LdotV - NdotL * NdotV;
    t            = t > 0.f ? t / fmaxf_(NdotL, NdotV) : 0.f;
    float sigma2 = sqr(roughness * kPi);
    float A      = 1.f - 0.5f * (sigma2 / (sigma2 + 0.33f));
    float B      = 0.45f * sigma2 / (sigma2 + 0.09f);
    return A + B * t;
}
AGB_DL v3 diffuseReflection(v3 L, v3 V, float weight, v3 color, float roughness, v3 N)
{
    if (weight < kFloatEps || !sameHemi(L, V, N))
        return splat(0.f);
    float NdotL = fmaxf_(dot(L, N), 0.f);
    v3 r        = divPi(color * weight * NdotL);
    if (roughness > 0.f)
        r *= orenNayar(L, V, N, NdotL, roughness);
    return r;
}
AGB_D float avgRoughness(v2 r) { return sqrtf(r.x * r.y); }
AGB_D float iorToF0(float ior) { return sqr((ior - 1.f) / (ior + 1.f)); }
AGB_D float mxNDF(v3 X, v3 Y, v3 H, float NdotH, float ax, float ay)
{
    float XdotH = dot(X, H);
    float YdotH = dot(Y, H);
    float denom = sqr(XdotH / ax) + sqr(YdotH / ay) + sqr(NdotH);
    return 1.f / (kPi * ax * ay * sqr(denom));
}
AGB_D float schlick(float cosTheta, float F0)
{
    float x = clampf(1.f - cosTheta, 0.f, 1.f);
    return F0 + (1.f - F0) * pow5(x);
}
AGB_D float smithG(float NdotL, float NdotV, float alpha)
{
    float a2 = sqr(alpha);
    float lL = sqrtf(a2 + (1.f - a2) * sqr(NdotL));
    float lV = sqrtf(a2 + (1.f - a2) * sqr(NdotV));
    return 2.f / (lL / NdotL + lV / NdotV);
}
// Curve-fit directional albedo; returns (AB.x, AB.y) so F0 * AB.x + F90 * AB.y.
AGB_D v2 dirAlbedoAB(float NdotV, float roughness)
{
    float r0 = roughness * -1.f + 1.f;
    float r1 = roughness * -0.0275f + 0.0425f;
    float r2 = roughness * -0.572f + 1.04f;
    float r3 = roughness * 0.022f + -0.04f;
    float a004 = fminf_(r0 * r0, agb_fm::exp2(-9.28f * NdotV)) * r0 + r1;
    return v2{ -1.04f * a004 + r2, 1.04f * a004 + r3 };
}
AGB_D float dirAlbedo(float NdotV, float roughness, float F0, float F90)
{
    v2 ab = dirAlbedoAB(NdotV, roughness);
    return F0 * ab.x + F90 * ab.y;
}
AGB_D float energyComp(float NdotV, float roughness, float Fss)
{
    float Ess = dirAlbedo(NdotV, roughness, 1.f, 1.f);
    return 1.f + Fss * (1.f - Ess) / Ess;
}
AGB_DL v3 energyComp3(float NdotV, float roughness, v3 Fss)
{
    float Ess = dirAlbedo(NdotV, roughness, 1.f, 1.f);
    return splat(1.f) + Fss * (1.f - Ess) / Ess;
}
AGB_DL v3 dielectricReflection(v3 L, v3 V, float weight, v3 tint, float ior, v2 rough, v3 N,
    v3 X, v3 base)
{
    if (weight < kFloatEps)
        return base;
    float NdotL = fabsf(dot(N, L));
    float NdotV = fabsf(dot(N, V));
    v3 Y        = normalize(cross(N, X));
    v3 H        = normalize(L + V);
    float NdotH = dot(N, H);
    float VdotH = dot(V, H);
    float avgR  = avgRoughness(rough);
    float F0    = iorToF0(ior);
    float D     = mxNDF(X, Y, H, NdotH, rough.x, rough.y);
    float F     = schlick(VdotH, F0);
    float G     = smithG(NdotL, NdotV, avgR);
    float comp  = energyComp(NdotV, avgR, F);
    float dA    = dirAlbedo(NdotV, avgR, F0, 1.f) * comp;
    v3 r        = abs3(tint * (D * F * G * comp) * weight / (4.f * NdotV));
    return r + base * (1.f - dA * weight);
}
AGB_D void artisticToComplexIOR(v3 reflectivity, v3 edge, v3& ior, v3& ext)
{
    v3 r     = clamp3(reflectivity, 0.f, 0.99f);
    v3 rs    = sqrt3(r);
    v3 nmin  = (splat(1.f) - r) / (splat(1.f) + r);
    v3 nmax  = (splat(1.f) + rs) / (splat(1.f) - rs);
    ior      = nmax + (nmin - nmax) * edge;
    v3 np1   = ior + splat(1.f);
    v3 nm1   = ior - splat(1.f);
    v3 k2    = (np1 * np1 * r - nm1 * nm1) / (splat(1.f) - r);
    ext      = sqrt3(max3(k2, 0.f));
}
AGB_D v3 fresnelConductor(float c, v3 n, v3 k)
{
    float c2 = c * c;
    v3 n2k2  = n * n + k * k;
    v3 nc2   = n * (2.f * c);
    v3 rsa   = n2k2 + splat(c2);
    v3 rpa   = n2k2 * c2 + splat(1.f);
    v3 rs    = (rsa - nc2) / (rsa + nc2);
    v3 rp    = (rpa - nc2) / (rpa + nc2);
    return (rs + rp) * 0.5f;
}
AGB_DL v3 conductorReflection(v3 L, v3 V, float weight, v3 refl, v3 edge, v2 rough, v3 N, v3 X)
{
    if (weight < kFloatEps || !sameHemi(L, V, N))
        return splat(0.f);
    float NdotL = fabsf(dot(N, L));
    float NdotV = fabsf(dot(N, V));
    v3 Y        = normalize(cross(N, X));
    v3 H        = normalize(L + V);
    float NdotH = dot(N, H);
    float VdotH = dot(V, H);
    v3 n, k;
    artisticToComplexIOR(refl, edge, n, k);
    float avgR = avgRoughness(rough);
    float D    = mxNDF(X, Y, H, NdotH, rough.x, rough.y);
    v3 F       = fresnelConductor(VdotH, n, k);
    float G    = smithG(NdotL, NdotV, avgR);
    v3 comp    = energyComp3(NdotV, avgR, F);
    return F * D * G * comp * weight / (4.f * NdotV);
}
AGB_D float sheenNDF(float cosTheta, float roughness)
{
    float inv  = 1.f / roughness;
    float sin2 = 1.f - cosTheta * cosTheta;
    return (2.f + inv) * agb_fm::pow(sin2, inv * 0.5f) / (2.f * kPi);
}
AGB_D float sheenAlbedo(float cosTheta, float roughness)
{
    float x = cosTheta * 15.f;
    float y = roughness * 15.f;
    int ix  = int(x);
    int iy  = int(y);
    int ix2 = min(max(ix + 1, 0), 15);
    int iy2 = min(max(iy + 1, 0), 15);
    float fx = x - float(ix);
    float fy = y - float(iy);
    float v1 = lerpf(agb_sheen_albedo_lut[iy * 16 + ix], agb_sheen_albedo_lut[iy * 16 + ix2], fx);
    float v2_ = lerpf(agb_sheen_albedo_lut[iy2 * 16 + ix], agb_sheen_albedo_lut[iy2 * 16 + ix2], fx);
    return clampf(lerpf(v1, v2_, fy), 0.f, 1.f);
}
AGB_DL v3 sheenReflection(v3 L, v3 V, float weight, v3 color, float roughness, v3 N, v3 base)
{
    if (weight < kFloatEps)
        return base;
    if (dot(N, V) < 0.f)
        N = -N;
    v3 H        = normalize(L + V);
    float NdotL = clampf(dot(N, L), kFloatEps, 1.f);
    float NdotV = clampf(dot(N, V), kFloatEps, 1.f);
    float NdotH = clampf(dot(N, H), kFloatEps, 1.f);
    float alpha = clampf(roughness, kFloatEps, 1.f);
    float D     = sheenNDF(NdotH, alpha);
    v3 fr       = color * D / (4.f * (NdotL + NdotV - NdotL * NdotV));
    float dA    = sheenAlbedo(NdotV, alpha);
    return fr * NdotL * weight + base * (1.f - dA * weight);
}
AGB_DL v3 sheenLayer(v3 L, v3 V, float weight, v3 color, float roughness, v3 N)
{
    if (!sameHemi(L, V, N))
        return splat(0.f);
    if (dot(N, V) < 0.f)
        N = -N;
    v3 H        = normalize(L + V);
    float NdotL = clampf(dot(N, L), kFloatEps, 1.f);
    float NdotV = clampf(dot(N, V), kFloatEps, 1.f);
    float NdotH = clampf(dot(N, H), kFloatEps, 1.f);
    float alpha = clampf(roughness, kFloatEps, 1.f);
    float D     = sheenNDF(NdotH, alpha);
    v3 fr       = color * D / (4.f * (NdotL + NdotV - NdotL * NdotV));
    return fr * NdotL * weight;
}
AGB_DL v3 subsurfaceReflection(v3 L, v3 V, float weight, v3 color, v3 N)
{
    float NdotL = dot(L, -N);
    if (NdotL <= 0.f || weight < kFloatEps)
        return splat(0.f);
    return divPi(color * weight * NdotL);
}
// mx_rotate_vector3 with HLSL row-major matrix construction (StandardSurfaceBSDF.slang:476-500).
AGB_D v3 rotateVector(v3 v, float degrees, v3 axis)
{
    if (degrees == 0.f)
        return v; // identity: cos 0 = 1, sin 0 = 0 reproduce v exactly
    float ang = degrees * (kPi / 180.f);
    axis      = normalize(axis);
    float s, c;
    agb_fm::sincos(ang, &s, &c);
    float oc = 1.f - c;
    v3 r0    = v3{ oc * axis.x * axis.x + c, oc * axis.x * axis.y - axis.z * s,
        oc * axis.z * axis.x + axis.y * s };
    v3 r1    = v3{ oc * axis.x * axis.y + axis.z * s, oc * axis.y * axis.y + c,
        oc * axis.y * axis.z - axis.x * s };
    v3 r2    = v3{ oc * axis.z * axis.x - axis.y * s, oc * axis.y * axis.z + axis.x * s,
        oc * axis.z * axis.z + c };
    return v3{ dot(r0, v), dot(r1, v), dot(r2, v) };
}
AGB_DL v3 dielectricDiffuseLayer(v3 L, v3 V, float weight, float ior, v2 rough, v3 N, v3 albedo)
{
    if (weight < kFloatEps || !sameHemi(L, V, N))
        return splat(0.f);
    float NdotV = fabsf(dot(N, V));
    v3 H        = normalize(L + V);
    float VdotH = dot(V, H);
    float avgR  = avgRoughness(rough);
    float F0    = iorToF0(ior);
    float F     = schlick(VdotH, F0);
    float comp  = energyComp(NdotV, avgR, F);
    float dA    = dirAlbedo(NdotV, avgR, F0, 1.f) * comp;
    return divPi(splat(1.f - dA) * albedo * weight);
}
AGB_DL v3 dielectricSpecularLayer(v3 L, v3 V, v3 tint, float ior, v2 rough, v3 N, v3 X)
{
    if (!sameHemi(L, V, N))
        return splat(0.f);
    float NdotL = fabsf(dot(N, L));
    float NdotV = fabsf(dot(N, V));
    v3 Y        = normalize(cross(N, X));
    v3 H        = normalize(L + V);
    float NdotH = dot(N, H);
    float VdotH = dot(V, H);
    float avgR  = avgRoughness(rough);
    float F0    = iorToF0(ior);
    float D     = mxNDF(X, Y, H, NdotH, rough.x, rough.y);
    float F     = schlick(VdotH, F0);
    float G     = smithG(NdotL, NdotV, avgR);
    float comp  = energyComp(NdotV, avgR, F);
    return abs3(tint * (D * F * G * comp) / (4.f * NdotV * NdotL));
}

// Values shared by the three Standard Surface entry points.
struct MatCommon
{
    v2 mainRough;
    v3 mainTangent;
    v3 coatTangent;
    v3 diffuseColor;    // coat-affected base color
    v3 subsurfaceColor; // coat-affected subsurface color
};
AGB_D MatCommon prepare(const Mat& m, const Frame& f)
{
    MatCommon c;
    float carf = m.coatAffectRoughness() * m.coat() * m.coatRoughness;
    float car  = lerpf(m.specularRoughness, 1.f, carf);
    float gamma = clampf(m.coat(), 0.f, 1.f) * m.coatAffectColor() + 1.f;
    c.subsurfaceColor = pow3(m.subsurfaceColor(), gamma);
    c.mainRough       = roughnessAniso(car, m.specularAnisotropy());
    c.mainTangent     = rotateVector(f.X, m.specularRotation() * 360.f, f.N);
    c.coatTangent     = rotateVector(f.X, m.coatRotation() * 360.f, f.N);
    c.diffuseColor    = pow3(m.baseColor, gamma);
    return c;
}

// evaluateMaterial (StandardSurfaceBSDF.slang:598-718): BSDF x cosine for world V, L.
AGB_DN v3 evaluateMaterial(const Mat& m, const MatCommon& c, const Frame& f, v3 Vw, v3 Lw)
{
    v3 dif      = diffuseReflection(Lw, Vw, m.base(), c.diffuseColor, m.diffuseRoughness(), f.N);
    v3 ssMix    = dif;
    if (m.subsurface() > 0.f)
        ssMix = mxMix(dif, subsurfaceReflection(Lw, Vw, 1.f, c.subsurfaceColor, f.N), m.subsurface());
    if (dot(f.N, Vw) * dot(f.N, Lw) < 0.f)
        return ssMix;
    v3 sd = ssMix;
    if (m.sheen() > 0.f)
        sd = sheenReflection(Lw, Vw, m.sheen(), m.sheenColor(), m.sheenRoughness(), f.N, ssMix);
    sd *= 1.f - m.transmission();
    v3 spec = sd;
    if (m.specular() > 0.f)
        spec = dielectricReflection(Lw, Vw, m.specular(), m.specularColor(), m.specularIOR(),
            c.mainRough, f.N, c.mainTangent, sd);
    v3 metalMix = spec;
    if (m.metalness() > 0.f)
    {
        v3 metal = conductorReflection(Lw, Vw, 1.f, m.metalColor() * m.base(),
            m.specularColor() * m.specular(), c.mainRough, f.N, c.mainTangent);
        metalMix = mxMix(spec, metal, m.metalness());
    }
    v3 fin = metalMix;
    if (m.coat() > 0.f)
    {
        v2 cr   = roughnessAniso(m.coatRoughness, m.coatAnisotropy());
        v3 att  = lerp3(splat(1.f), m.coatColor(), m.coat());
        fin     = dielectricReflection(Lw, Vw, m.coat(), m.coatColor(), m.coatIOR(), cr, f.N,
            c.coatTangent, att * metalMix);
    }
    return fin;
}

AGB_D float ggxPdfForL(v3 V, v2 alpha, v3 L)
{
    v3 H = normalize(V + L);
    return ggxVNDF(V, H, alpha) / (4.f * dot(V, H));
}
AGB_DL v3 sampleGGXLight(const Frame& f, v3 V, v2 alpha, v2 r, v3& Lw, float& pdf)
{
    bool flip = V.z <= 0.f;
    v3 H      = sampleGGXVNDF(flip ? -V : V, alpha, r);
    H         = flip ? -H : H;
    v3 L      = reflect(-V, H);
    pdf       = ggxVNDF(V, H, alpha) / (4.f * dot(V, H));
    Lw        = toWorld(L, f);
    return L;
}
AGB_D v3 sampleHemiTangent(v3 V, v2 r, float& pdf)
{
    return sampleHemisphereAbout(r, v3{ 0.f, 0.f, V.z > 0.f ? 1.f : -1.f }, pdf);
}
AGB_DL v3 computeRefraction(v3 V, float ior, bool& reflected)
{
    reflected     = false;
    bool entering = V.z > 0.f;
    v3 N          = v3{ 0.f, 0.f, entering ? 1.f : -1.f };
    float eta     = entering ? 1.f / ior : ior / 1.f;
    v3 L          = refract(-V, N, eta);
    if (length(L) == 0.f)
    {
        L         = v3{ -V.x, -V.y, V.z };
        reflected = true;
    }
    return L;
}

// evaluateMaterialAndPDF (StandardSurfaceBSDF.slang:862-1088).
AGB_DN v3 evaluateMaterialAndPDF(const Mat& m, const MatCommon& c, const Frame& f, v3 Vw, v3 Lw, v2 rnd, float& pdf,
    int& lobe)
{
    v3 V        = toTangent(Vw, f);
    v3 L        = toTangent(Lw, f);
    float NdotV = fabsf(V.z);
    pdf         = 0.f;
    lobe        = NO_SECONDARY_RAY;
    v3 result;
    float coatLum = luminance(splat(schlick(NdotV, iorToF0(m.coatIOR()))) * m.coat() * m.coatColor());
    if (rnd.x < coatLum)
    {
        v2 ca  = roughnessAniso(m.coatRoughness, m.coatAnisotropy());
        pdf    = ggxPdfForL(V, ca, L);
        result = dielectricSpecularLayer(Lw, Vw, m.coatColor() * m.coat(), m.coatIOR(), ca, f.N,
            c.coatTangent);
        lobe   = COAT_LOBE;
    }
    else
    {
        rnd.x   = (rnd.x - coatLum) / (1.f - coatLum);
        v2 sa   = roughnessAniso(m.specularRoughness, m.specularAnisotropy());
        if (rnd.x < m.metalness())
        {
            pdf    = ggxPdfForL(V, sa, L);
            result = conductorReflection(Lw, Vw, 1.f, m.metalColor() * m.base(),
                m.specularColor() * m.specular(), c.mainRough, f.N, c.mainTangent);
            result /= fabsf(L.z);
            lobe = METAL_LOBE;
        }
        else
        {
            rnd.x          = (rnd.x - m.metalness()) / (1.f - m.metalness());
            float specLum  = luminance(
                splat(schlick(NdotV, iorToF0(m.specularIOR()))) * m.specular() * m.specularColor());
            if (rnd.x < specLum)
            {
                pdf    = ggxPdfForL(V, sa, L);
                result = dielectricSpecularLayer(Lw, Vw, m.specularColor() * m.specular(),
                    m.specularIOR(), c.mainRough, f.N, c.mainTangent);
                result /= specLum;
                lobe = GLOSSY_LOBE;
            }
            else
            {
                rnd.x            = (rnd.x - specLum) / (1.f - specLum);
                float sheenAlpha = clampf(m.sheenRoughness(), kFloatEps, 1.f);
                if (rnd.x < m.sheen())
                {
                    v3 H   = normalize(L + V);
                    result = sheenLayer(Lw, Vw, m.sheen(), m.sheenColor(), m.sheenRoughness(), f.N);
                    pdf    = sheenNDF(H.z, sheenAlpha);
                    lobe   = SHEEN_LOBE;
                }
                else
                {
                    pdf    = divPi(dot(f.N, Lw));
                    result = dielectricDiffuseLayer(Lw, Vw, m.base(), m.specularIOR(), c.mainRough,
                        f.N, c.diffuseColor);
                    result *= (1.f - sheenAlbedo(NdotV, sheenAlpha) * m.sheen());
                    lobe = DIFFUSE_LOBE;
                }
            }
        }
        result *= lerp3(splat(1.f), m.coatColor(), m.coat());
    }
    return result * fabsf(L.z);
}

// sampleMaterial (StandardSurfaceBSDF.slang:1093-1372).
AGB_DN v3 sampleMaterial(const Mat& m, const MatCommon& c, const Frame& f, v3 Vw, v2 rnd, v3& Lw, float& pdf,
    int& lobe)
{
    v3 L;
    v3 V        = toTangent(Vw, f);
    float NdotV = fabsf(V.z);
    Lw          = v3{ 1.f, 0.f, 0.f };
    pdf         = 0.f;
    lobe        = NO_SECONDARY_RAY;
    v3 result;
    float coatLum = luminance(splat(schlick(NdotV, iorToF0(m.coatIOR()))) * m.coat() * m.coatColor());
    if (rnd.x < coatLum)
    {
        rnd.x  = rnd.x / coatLum;
        v2 ca  = roughnessAniso(m.coatRoughness, m.coatAnisotropy());
        L      = sampleGGXLight(f, V, ca, rnd, Lw, pdf);
        result = dielectricSpecularLayer(Lw, Vw, m.coatColor() * m.coat(), m.coatIOR(), ca, f.N,
            c.coatTangent);
        result /= coatLum;
        lobe = COAT_LOBE;
    }
    else
    {
        rnd.x = (rnd.x - coatLum) / (1.f - coatLum);
        v2 sa = roughnessAniso(m.specularRoughness, m.specularAnisotropy());
        if (rnd.x < m.metalness())
        {
            rnd.x  = rnd.x / m.metalness();
            L      = sampleGGXLight(f, V, sa, rnd, Lw, pdf);
            result = conductorReflection(Lw, Vw, 1.f, m.metalColor() * m.base(),
                m.specularColor() * m.specular(), c.mainRough, f.N, c.mainTangent);
            result /= fabsf(L.z);
            lobe = METAL_LOBE;
        }
        else
        {
            rnd.x         = (rnd.x - m.metalness()) / (1.f - m.metalness());
            float specLum = luminance(
                splat(schlick(NdotV, iorToF0(m.specularIOR()))) * m.specular() * m.specularColor());
            if (rnd.x < specLum)
            {
                rnd.x  = rnd.x / specLum;
                L      = sampleGGXLight(f, V, sa, rnd, Lw, pdf);
                result = dielectricSpecularLayer(Lw, Vw, m.specularColor() * m.specular(),
                    m.specularIOR(), c.mainRough, f.N, c.mainTangent);
                result /= specLum;
                lobe = GLOSSY_LOBE;
            }
            else
            {
                rnd.x            = (rnd.x - specLum) / (1.f - specLum);
                float sheenAlpha = clampf(m.sheenRoughness(), kFloatEps, 1.f);
                if (rnd.x < m.sheen())
                {
                    rnd.x  = rnd.x / m.sheen();
                    L      = sampleHemiTangent(V, rnd, pdf);
                    Lw     = toWorld(L, f);
                    v3 H   = normalize(L + V);
                    result = sheenLayer(Lw, Vw, m.sheen(), m.sheenColor(), m.sheenRoughness(), f.N);
                    pdf    = sheenNDF(H.z, sheenAlpha);
                    lobe   = SHEEN_LOBE;
                }
                else
                {
                    rnd.x = (rnd.x - m.sheen()) / (1.f - m.sheen());
                    if (rnd.x < m.transmission())
                    {
                        bool reflected = false;
                        L              = -V;
                        if (!m.thinWalled())
                            L = computeRefraction(V, m.specularIOR(), reflected);
                        Lw     = toWorld(L, f);
                        result = m.transmissionColor();
                        result /= fabsf(L.z);
                        pdf  = 1.f;
                        lobe = reflected ? GLOSSY_LOBE : TRANSMISSION_LOBE;
                    }
                    else
                    {
                        rnd.x  = (rnd.x - m.transmission()) / (1.f - m.transmission());
                        L      = sampleHemiTangent(V, rnd, pdf);
                        Lw     = toWorld(L, f);
                        result = dielectricDiffuseLayer(Lw, Vw, m.base(), m.specularIOR(),
                            c.mainRough, f.N, c.diffuseColor);
                        result *= (1.f - sheenAlbedo(NdotV, sheenAlpha) * m.sheen());
                        lobe = DIFFUSE_LOBE;
                    }
                }
            }
        }
        result *= lerp3(splat(1.f), m.coatColor(), m.coat());
    }
    return result * fabsf(L.z);
}

// The entry points with the shared values computed for the call (one shading point, one call).
AGB_D v3 evaluateMaterial(const Mat& m, const Frame& f, v3 Vw, v3 Lw)
{
    return evaluateMaterial(m, prepare(m, f), f, Vw, Lw);
}
AGB_D v3 evaluateMaterialAndPDF(const Mat& m, const Frame& f, v3 Vw, v3 Lw, v2 rnd, float& pdf, int& lobe)
{
    return evaluateMaterialAndPDF(m, prepare(m, f), f, Vw, Lw, rnd, pdf, lobe);
}
AGB_D v3 sampleMaterial(const Mat& m, const Frame& f, v3 Vw, v2 rnd, v3& Lw, float& pdf, int& lobe)
{
    return sampleMaterial(m, prepare(m, f), f, Vw, rnd, Lw, pdf, lobe);
}

} // namespace agb
