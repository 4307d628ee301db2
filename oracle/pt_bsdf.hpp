// Oracle (test infrastructure, never linked into the product): CPU restatement of Aurora's
// Standard Surface BSDF and its sampling helpers, templated on the scalar type.
//
// Follows, function for function and in the same operation order:
//   Shaders/Sampling.slang:20-107        (uniform / cosine hemisphere / cone / disk, MIS weight)
//   Shaders/Globals.slang:47-69          (buildBasis)
//   Shaders/BSDFCommon.slang:76-299      (remap, tangent frames, refraction, GGX VNDF)
//   Shaders/StandardSurfaceBSDF.slang:22-1372 (mx_* lobes, evaluateMaterial,
//                                          evaluateMaterialAndPDF, sampleMaterial)
// with the non-denoising lobe selection (getGlossySelectionProbability returns specLuminance and
// getNonGlossyLobeCompensation returns 1, StandardSurfaceBSDF.slang:193-235).
//
// Note on M_PI_INV: the reference macro is `1.0 / 3.14159...` without parentheses, so `x * M_PI_INV`
// is `(x * 1.0) / pi`, a division.  divPi() restates that.
#pragma once

#include "pt_math.hpp"
#include "sheen_lut.hpp"

namespace orc
{

// Lobe and ray-type identifiers (Shaders/BSDFCommon.slang:28-39).
enum : int
{
    TRANSPARENCY_LOBE          = 1,
    COAT_LOBE                  = 2,
    METAL_LOBE                 = 3,
    GLOSSY_LOBE                = 4,
    TRANSMISSION_LOBE          = 5,
    SHEEN_LOBE                 = 6,
    DIFFUSE_LOBE               = 7,
    NO_SECONDARY_RAY           = 8,
    CAMERA_RAY                 = 9,
    GROUND_PLANE_REFLECTION_RAY = 10
};

// Material values used during evaluation (Shaders/Material.slang:20-57).
template <class T>
struct Material
{
    T base;
    V3<T> baseColor;
    T diffuseRoughness;
    T metalness;
    V3<T> metalColor;
    T specular;
    V3<T> specularColor;
    T specularRoughness;
    T specularIOR;
    T specularAnisotropy;
    T specularRotation;
    T transmission;
    V3<T> transmissionColor;
    T subsurface;
    V3<T> subsurfaceColor;
    V3<T> subsurfaceRadius;
    T subsurfaceScale;
    T subsurfaceAnisotropy;
    T sheen;
    V3<T> sheenColor;
    T sheenRoughness;
    T coat;
    V3<T> coatColor;
    T coatRoughness;
    T coatAnisotropy;
    T coatRotation;
    T coatIOR;
    T coatAffectColor;
    T coatAffectRoughness;
    T emission;
    V3<T> emissionColor;
    V3<T> opacity;
    bool thinWalled;
};

// The subset of ShadingData (Shaders/Geometry.slang:29-89) that the default material uses.
template <class T>
struct ShadingData
{
    V3<T> normal;
    V3<T> tangent;
    V3<T> bitangent;
    V3<T> position;
    V3<T> geomPosition;
    V2<T> texCoord;
    uint32_t indices[3] = { 0, 0, 0 };
    V3<T> barycentrics;
};

template <class T>
struct BSDF
{
    using v2 = V2<T>;
    using v3 = V3<T>;
    static constexpr T PI  = Consts<T>::PI;
    static constexpr T EPS = Consts<T>::FLOAT_EPS;

    static T divPi(T x) { return (x * T(1)) / PI; }
    static v3 divPi(const v3& x) { return (x * T(1)) / PI; }
    static T sqr(T x) { return x * x; }
    static T fmin_(T a, T b) { return a < b ? a : b; }
    static T fmax_(T a, T b) { return a > b ? a : b; }

    // ---------------------------------------------------------------------------------- Sampling
    // Sampling.slang:20-32
    static v3 sampleUniformDirection(v2 random, T& pdf)
    {
        T cosTheta = T(1) - T(2) * random[1];
        T sinTheta = std::sqrt(T(1) - cosTheta * cosTheta);
        T phi      = T(2) * PI * random[0];
        v3 dir(sinTheta * tcos(phi), sinTheta * tsin(phi), cosTheta);
        pdf = divPi(T(0.25f));
        return dir;
    }
    // Sampling.slang:37-49 (cosine hemisphere about an arbitrary normal)
    static v3 sampleHemisphere(v2 random, const v3& normal, T& pdf)
    {
        v3 direction = sampleUniformDirection(random, pdf);
        direction    = normalize(normal + direction);
        pdf          = divPi(dot(normal, direction));
        return direction;
    }
    // Globals.slang:47-52
    static void buildBasis(const v3& normal, v3& tangent, v3& bitangent)
    {
        bitangent = std::fabs(normal.y) < T(0.999f) ? v3(0, 1, 0) : v3(1, 0, 0);
        tangent   = normalize(cross(bitangent, normal));
        bitangent = cross(normal, tangent);
    }
    // Sampling.slang:69-83
    static v3 sampleCone(v2 random, const v3& direction, T cosThetaMax)
    {
        v3 xb, yb;
        buildBasis(direction, xb, yb);
        T cosTheta = (T(1) - random[0]) + random[0] * cosThetaMax;
        T sinTheta = std::sqrt(T(1) - cosTheta * cosTheta);
        T phi      = random[1] * T(2) * PI;
        return xb * tcos(phi) * sinTheta + yb * tsin(phi) * sinTheta + direction * cosTheta;
    }
    // Sampling.slang:87-93
    static v2 sampleDisk(v2 random, T radius)
    {
        T r   = radius * std::sqrt(random[0]);
        T phi = T(2) * PI * random[1];
        return v2(tcos(phi), tsin(phi)) * r;
    }
    // Sampling.slang:98-104 (power heuristic with n = 1)
    static T computeMISWeight(T fPDF, T gPDF)
    {
        T f = T(1) * fPDF;
        T g = T(1) * gPDF;
        return (f * f) / (f * f + g * g);
    }

    // ------------------------------------------------------------------------------ BSDFCommon
    static T remapPass(T r, T test) { return r / test; }
    static T remapFail(T r, T test) { return (r - test) / (T(1) - test); }
    static v3 worldToTangent(const v3& i, const v3& X, const v3& Y, const v3& N)
    {
        return v3(dot(i, X), dot(i, Y), dot(i, N));
    }
    static v3 tangentToWorld(const v3& i, const v3& X, const v3& Y, const v3& N)
    {
        return X * i.x + Y * i.y + N * i.z;
    }
    // BSDFCommon.slang:122-152
    static v3 computeRefraction(const v3& V, T ior, bool& reflected)
    {
        reflected         = false;
        bool entering     = V.z > T(0);
        v3 N(0, 0, entering ? T(1) : T(-1));
        T eta = entering ? T(1) / ior : ior / T(1);
        v3 L  = refract(-V, N, eta);
        if (length(L) == T(0))
        {
            L         = v3(-V.x, -V.y, V.z);
            reflected = true;
        }
        return L;
    }
    // BSDFCommon.slang:208-213
    static T lambda(const v3& vec, v2 alpha)
    {
        T squared = (sqr(alpha.x) * sqr(vec.x) + sqr(alpha.y) * sqr(vec.y)) / sqr(vec.z);
        return (T(-1) + std::sqrt(T(1) + squared)) * T(0.5f);
    }
    static T evaluateSmithG1(const v3& V, const v3& H, v2 alpha)
    {
        if (dot(V, H) <= T(0))
            return T(0);
        return T(1) / (T(1) + lambda(V, alpha));
    }
    static T evaluateGGXNDF(const v3& H, v2 alpha)
    {
        T ellipse = sqr(H.x) / sqr(alpha.x) + sqr(H.y) / sqr(alpha.y) + sqr(H.z);
        return T(1) / (PI * alpha.x * alpha.y * sqr(ellipse));
    }
    static T evaluateGGXSmithVNDF(const v3& V, const v3& H, v2 alpha)
    {
        T VDotH = dot(V, H);
        if (VDotH <= T(0))
            return T(0);
        T D  = evaluateGGXNDF(H, alpha);
        T G1 = evaluateSmithG1(V, H, alpha);
        return D * G1 * VDotH / std::fabs(V.z);
    }
    // BSDFCommon.slang:274-299
    static v3 sampleGGXSmithVNDF(const v3& V, v2 alpha, v2 random)
    {
        v3 Vh    = normalize(v3(alpha.x * V.x, alpha.y * V.y, V.z));
        T lensq  = Vh.x * Vh.x + Vh.y * Vh.y;
        v3 T1    = lensq > T(0) ? v3(-Vh.y, Vh.x, T(0)) / std::sqrt(lensq) : v3(1, 0, 0);
        v3 T2    = cross(Vh, T1);
        T r      = std::sqrt(random.x);
        T phi    = T(2) * PI * random.y;
        T t1     = r * tcos(phi);
        T t2     = r * tsin(phi);
        T s      = T(0.5f) * (T(1) + Vh.z);
        t2       = (T(1) - s) * std::sqrt(T(1) - t1 * t1) + s * t2;
        v3 Nh    = T1 * t1 + T2 * t2 + Vh * std::sqrt(fmax_(T(0), T(1) - t1 * t1 - t2 * t2));
        return normalize(v3(alpha.x * Nh.x, alpha.y * Nh.y, fmax_(T(0), Nh.z)));
    }

    // ----------------------------------------------------------------------- MaterialX helpers
    static bool sameHemisphere(const v3& a, const v3& b, const v3& n)
    {
        return dot(a, n) * dot(b, n) > T(0);
    }
    static v2 mx_roughness_anisotropy(T roughness, T anisotropy)
    {
        v2 result;
        T rsq = clampT(roughness * roughness, EPS, T(1));
        if (anisotropy > T(0))
        {
            T aspect = std::sqrt(T(1) - clampT(anisotropy, T(0), T(0.98f)));
            result.x = fmin_(rsq / aspect, T(1));
            result.y = rsq * aspect;
        }
        else
        {
            result.x = rsq;
            result.y = rsq;
        }
        return result;
    }
    static T mx_pow5(T x) { return sqr(sqr(x)) * x; }
    static v3 mx_mix(const v3& bg, const v3& fg, T w) { return lerp(bg, fg, clampT(w, T(0), T(1))); }
    static T mx_orennayar(const v3& L, const v3& V, const v3& N, T NdotL, T roughness)
    {
        T LdotV  = dot(L, V);
        T NdotV  = std::fabs(dot(N, V));
        T t      = LdotV - NdotL * NdotV;
        t        = t > T(0) ? t / fmax_(NdotL, NdotV) : T(0);
        T sigma2 = sqr(roughness * PI);
        T A      = T(1) - T(0.5f) * (sigma2 / (sigma2 + T(0.33f)));
        T B      = T(0.45f) * sigma2 / (sigma2 + T(0.09f));
        return A + B * t;
    }
    static v3 mx_diffuse_brdf_reflection(
        const v3& L, const v3& V, T weight, const v3& color, T roughness, const v3& normal)
    {
        if (weight < EPS || !sameHemisphere(L, V, normal))
            return v3(0);
        T NdotL   = fmax_(dot(L, normal), T(0));
        v3 result = divPi(color * weight * NdotL);
        if (roughness > T(0))
            result *= mx_orennayar(L, V, normal, NdotL, roughness);
        return result;
    }
    static T mx_average_roughness(v2 r) { return std::sqrt(r.x * r.y); }
    static T mx_ior_to_f0(T ior) { return sqr((ior - T(1)) / (ior + T(1))); }
    static T mx_ggx_NDF(const v3& X, const v3& Y, const v3& H, T NdotH, T ax, T ay)
    {
        T XdotH = dot(X, H);
        T YdotH = dot(Y, H);
        T denom = sqr(XdotH / ax) + sqr(YdotH / ay) + sqr(NdotH);
        return T(1) / (PI * ax * ay * sqr(denom));
    }
    static T mx_fresnel_schlick(T cosTheta, T F0)
    {
        T x  = clampT(T(1) - cosTheta, T(0), T(1));
        T x5 = mx_pow5(x);
        return F0 + (T(1) - F0) * x5;
    }
    static T mx_ggx_smith_G(T NdotL, T NdotV, T alpha)
    {
        T alpha2  = sqr(alpha);
        T lambdaL = std::sqrt(alpha2 + (T(1) - alpha2) * sqr(NdotL));
        T lambdaV = std::sqrt(alpha2 + (T(1) - alpha2) * sqr(NdotV));
        return T(2) / (lambdaL / NdotL + lambdaV / NdotV);
    }
    static v3 mx_ggx_directional_albedo_curve_fit(T NdotV, T roughness, const v3& F0, const v3& F90)
    {
        const T c0[4] = { T(-1), T(-0.0275f), T(-0.572f), T(0.022f) };
        const T c1[4] = { T(1), T(0.0425f), T(1.04f), T(-0.04f) };
        T r[4];
        for (int i = 0; i < 4; i++)
            r[i] = roughness * c0[i] + c1[i];
        T a004 = fmin_(r[0] * r[0], texp2(T(-9.28f) * NdotV)) * r[0] + r[1];
        T ABx  = T(-1.04f) * a004 + r[2];
        T ABy  = T(1.04f) * a004 + r[3];
        return F0 * ABx + F90 * ABy;
    }
    static T mx_ggx_directional_albedo(T NdotV, T roughness, T F0, T F90)
    {
        return mx_ggx_directional_albedo_curve_fit(NdotV, roughness, v3(F0), v3(F90)).x;
    }
    static v3 mx_ggx_energy_compensation(T NdotV, T roughness, const v3& Fss)
    {
        T Ess = mx_ggx_directional_albedo(NdotV, roughness, T(1), T(1));
        return v3(T(1)) + Fss * (T(1) - Ess) / Ess;
    }
    static T mx_ggx_energy_compensation(T NdotV, T roughness, T Fss)
    {
        return mx_ggx_energy_compensation(NdotV, roughness, v3(Fss)).x;
    }
    static v3 mx_dielectric_brdf_reflection(const v3& L, const v3& V, T weight, const v3& tint,
        T ior, v2 roughness, const v3& N, const v3& X, const v3& base)
    {
        if (weight < EPS)
            return base;
        T NdotL       = std::fabs(dot(N, L));
        T NdotV       = std::fabs(dot(N, V));
        v3 Y          = normalize(cross(N, X));
        v3 H          = normalize(L + V);
        T NdotH       = dot(N, H);
        T VdotH       = dot(V, H);
        T avgR        = mx_average_roughness(roughness);
        T F0          = mx_ior_to_f0(ior);
        T D           = mx_ggx_NDF(X, Y, H, NdotH, roughness.x, roughness.y);
        T F           = mx_fresnel_schlick(VdotH, F0);
        T G           = mx_ggx_smith_G(NdotL, NdotV, avgR);
        T comp        = mx_ggx_energy_compensation(NdotV, avgR, F);
        T dirAlbedo   = mx_ggx_directional_albedo(NdotV, avgR, F0, T(1)) * comp;
        v3 result     = abs3(tint * (D * F * G * comp) * weight / (T(4) * NdotV));
        result += base * (T(1) - dirAlbedo * weight);
        return result;
    }
    static void mx_artistic_to_complex_ior(
        const v3& reflectivity, const v3& edge_color, v3& ior, v3& extinction)
    {
        v3 r      = clamp3(reflectivity, T(0), T(0.99f));
        v3 r_sqrt = sqrt3(r);
        v3 n_min  = (v3(1) - r) / (v3(1) + r);
        v3 n_max  = (v3(1) + r_sqrt) / (v3(1) - r_sqrt);
        ior       = n_max + (n_min - n_max) * edge_color;
        v3 np1    = ior + v3(1);
        v3 nm1    = ior - v3(1);
        v3 k2     = (np1 * np1 * r - nm1 * nm1) / (v3(1) - r);
        k2        = max3(k2, T(0));
        extinction = sqrt3(k2);
    }
    static v3 mx_fresnel_conductor(T cosTheta, const v3& n, const v3& k)
    {
        T c2     = cosTheta * cosTheta;
        v3 n2_k2 = n * n + k * k;
        v3 nc2   = n * (T(2) * cosTheta);
        v3 rs_a  = n2_k2 + v3(c2);
        v3 rp_a  = n2_k2 * c2 + v3(1);
        v3 rs    = (rs_a - nc2) / (rs_a + nc2);
        v3 rp    = (rp_a - nc2) / (rp_a + nc2);
        return (rs + rp) * T(0.5f);
    }
    static v3 mx_conductor_brdf_reflection(const v3& L, const v3& V, T weight,
        const v3& reflectivity, const v3& edge_color, v2 roughness, const v3& N, const v3& X)
    {
        if (weight < EPS || !sameHemisphere(L, V, N))
            return v3(0);
        T NdotL = std::fabs(dot(N, L));
        T NdotV = std::fabs(dot(N, V));
        v3 Y    = normalize(cross(N, X));
        v3 H    = normalize(L + V);
        T NdotH = dot(N, H);
        T VdotH = dot(V, H);
        v3 ior_n, ior_k;
        mx_artistic_to_complex_ior(reflectivity, edge_color, ior_n, ior_k);
        T avgR  = mx_average_roughness(roughness);
        T D     = mx_ggx_NDF(X, Y, H, NdotH, roughness.x, roughness.y);
        v3 F    = mx_fresnel_conductor(VdotH, ior_n, ior_k);
        T G     = mx_ggx_smith_G(NdotL, NdotV, avgR);
        v3 comp = mx_ggx_energy_compensation(NdotV, avgR, F);
        return F * D * G * comp * weight / (T(4) * NdotV);
    }
    static T mx_imageworks_sheen_NDF(T cosTheta, T roughness)
    {
        T invR = T(1) / roughness;
        T cos2 = cosTheta * cosTheta;
        T sin2 = T(1) - cos2;
        return (T(2) + invR) * tpow(sin2, invR * T(0.5f)) / (T(2) * PI);
    }
    static T mx_imageworks_sheen_directional_albedo(T cosTheta, T roughness)
    {
        T x    = cosTheta * T(15);
        T y    = roughness * T(15);
        int ix = int(x);
        int iy = int(y);
        int ix2 = ix + 1 < 0 ? 0 : (ix + 1 > 15 ? 15 : ix + 1);
        int iy2 = iy + 1 < 0 ? 0 : (iy + 1 > 15 ? 15 : iy + 1);
        T fx   = x - T(ix);
        T fy   = y - T(iy);
        T v1   = lerp(T(kSheenAlbedoLUT[iy * 16 + ix]), T(kSheenAlbedoLUT[iy * 16 + ix2]), fx);
        T v2   = lerp(T(kSheenAlbedoLUT[iy2 * 16 + ix]), T(kSheenAlbedoLUT[iy2 * 16 + ix2]), fx);
        return clampT(lerp(v1, v2, fy), T(0), T(1));
    }
    static v3 mx_sheen_brdf_reflection(const v3& L, const v3& V, T weight, const v3& color,
        T roughness, v3 N, const v3& base)
    {
        if (weight < EPS)
            return base;
        if (dot(N, V) < T(0))
            N = -N;
        v3 H      = normalize(L + V);
        T NdotL   = clampT(dot(N, L), EPS, T(1));
        T NdotV   = clampT(dot(N, V), EPS, T(1));
        T NdotH   = clampT(dot(N, H), EPS, T(1));
        T alpha   = clampT(roughness, EPS, T(1));
        T D       = mx_imageworks_sheen_NDF(NdotH, alpha);
        v3 fr     = color * D / (T(4) * (NdotL + NdotV - NdotL * NdotV));
        T dirAlb  = mx_imageworks_sheen_directional_albedo(NdotV, alpha);
        return fr * NdotL * weight + base * (T(1) - dirAlb * weight);
    }
    static v3 mx_sheen_brdf_specular_layer(
        const v3& L, const v3& V, T weight, const v3& color, T roughness, v3 N)
    {
        if (!sameHemisphere(L, V, N))
            return v3(0);
        if (dot(N, V) < T(0))
            N = -N;
        v3 H    = normalize(L + V);
        T NdotL = clampT(dot(N, L), EPS, T(1));
        T NdotV = clampT(dot(N, V), EPS, T(1));
        T NdotH = clampT(dot(N, H), EPS, T(1));
        T alpha = clampT(roughness, EPS, T(1));
        T D     = mx_imageworks_sheen_NDF(NdotH, alpha);
        v3 fr   = color * D / (T(4) * (NdotL + NdotV - NdotL * NdotV));
        return fr * NdotL * weight;
    }
    static v3 mx_subsurface_brdf_reflection(
        const v3& L, const v3& V, T weight, const v3& color, const v3& normal)
    {
        T NdotL = dot(L, -normal);
        if (NdotL <= T(0) || weight < EPS)
            return v3(0);
        return divPi(color * weight * NdotL);
    }
    // mx_rotate_vector3 with the HLSL row-major float4x4 constructor (StandardSurfaceBSDF.slang:476-500).
    static v3 mx_rotate_vector3(const v3& vec, T amountDegrees, v3 axis)
    {
        T angle = amountDegrees * (PI / T(180));
        axis    = normalize(axis);
        T s     = tsin(angle);
        T c     = tcos(angle);
        T oc    = T(1) - c;
        T r0[3] = { oc * axis.x * axis.x + c, oc * axis.x * axis.y - axis.z * s,
            oc * axis.z * axis.x + axis.y * s };
        T r1[3] = { oc * axis.x * axis.y + axis.z * s, oc * axis.y * axis.y + c,
            oc * axis.y * axis.z - axis.x * s };
        T r2[3] = { oc * axis.z * axis.x - axis.y * s, oc * axis.y * axis.z + axis.x * s,
            oc * axis.z * axis.z + c };
        return v3(r0[0] * vec.x + r0[1] * vec.y + r0[2] * vec.z + T(0),
            r1[0] * vec.x + r1[1] * vec.y + r1[2] * vec.z + T(0),
            r2[0] * vec.x + r2[1] * vec.y + r2[2] * vec.z + T(0));
    }
    static v3 mx_dielectric_brdf_diffuse_layer(const v3& L, const v3& V, T weight, T ior,
        v2 roughness, const v3& N, const v3& albedo)
    {
        if (weight < EPS || !sameHemisphere(L, V, N))
            return v3(0);
        T NdotV     = std::fabs(dot(N, V));
        v3 H        = normalize(L + V);
        T VdotH     = dot(V, H);
        T avgR      = mx_average_roughness(roughness);
        T F0        = mx_ior_to_f0(ior);
        T F         = mx_fresnel_schlick(VdotH, F0);
        T comp      = mx_ggx_energy_compensation(NdotV, avgR, F);
        T dirAlbedo = mx_ggx_directional_albedo(NdotV, avgR, F0, T(1)) * comp;
        v3 result   = v3(T(1) - dirAlbedo);
        return divPi(result * albedo * weight);
    }
    static v3 mx_dielectric_brdf_specular_layer(const v3& L, const v3& V, const v3& tint, T ior,
        v2 roughness, const v3& N, const v3& X)
    {
        if (!sameHemisphere(L, V, N))
            return v3(0);
        T NdotL = std::fabs(dot(N, L));
        T NdotV = std::fabs(dot(N, V));
        v3 Y    = normalize(cross(N, X));
        v3 H    = normalize(L + V);
        T NdotH = dot(N, H);
        T VdotH = dot(V, H);
        T avgR  = mx_average_roughness(roughness);
        T F0    = mx_ior_to_f0(ior);
        T D     = mx_ggx_NDF(X, Y, H, NdotH, roughness.x, roughness.y);
        T F     = mx_fresnel_schlick(VdotH, F0);
        T G     = mx_ggx_smith_G(NdotL, NdotV, avgR);
        T comp  = mx_ggx_energy_compensation(NdotV, avgR, F);
        return abs3(tint * (D * F * G * comp) / (T(4) * NdotV * NdotL));
    }

    // --------------------------------------------------------------------- Standard Surface
    struct Common
    {
        v2 main_roughness;
        v3 main_tangent;
        v3 coat_tangent;
        v3 coat_affected_diffuse_color;
        v3 coat_affected_subsurface_color;
    };
    static Common prepare(const Material<T>& m, const ShadingData<T>& sh)
    {
        Common c;
        T coat_affect_roughness_factor = m.coatAffectRoughness * m.coat * m.coatRoughness;
        T coat_affected_roughness = lerp(m.specularRoughness, T(1), coat_affect_roughness_factor);
        T coat_clamped            = clampT(m.coat, T(0), T(1));
        T coat_gamma              = coat_clamped * m.coatAffectColor + T(1);
        c.coat_affected_subsurface_color = pow3(m.subsurfaceColor, coat_gamma);
        c.main_roughness = mx_roughness_anisotropy(coat_affected_roughness, m.specularAnisotropy);
        c.main_tangent   = mx_rotate_vector3(sh.tangent, m.specularRotation * T(360), sh.normal);
        c.coat_tangent   = mx_rotate_vector3(sh.tangent, m.coatRotation * T(360), sh.normal);
        c.coat_affected_diffuse_color = pow3(m.baseColor, coat_gamma);
        return c;
    }

    // StandardSurfaceBSDF.slang:598-718
    static v3 evaluateMaterial(const Material<T>& m, const ShadingData<T>& sh, const v3& Vw,
        const v3& Lw)
    {
        Common c        = prepare(m, sh);
        v3 diffuse_bsdf = mx_diffuse_brdf_reflection(
            Lw, Vw, m.base, c.coat_affected_diffuse_color, m.diffuseRoughness, sh.normal);
        v3 subsurface_mix = diffuse_bsdf;
        if (m.subsurface > T(0))
        {
            v3 ss = mx_subsurface_brdf_reflection(
                Lw, Vw, T(1), c.coat_affected_subsurface_color, sh.normal);
            subsurface_mix = mx_mix(diffuse_bsdf, ss, m.subsurface);
        }
        if (dot(sh.normal, Vw) * dot(sh.normal, Lw) < T(0))
            return subsurface_mix;
        v3 sheen_and_diffuse = subsurface_mix;
        if (m.sheen > T(0))
            sheen_and_diffuse = mx_sheen_brdf_reflection(
                Lw, Vw, m.sheen, m.sheenColor, m.sheenRoughness, sh.normal, subsurface_mix);
        sheen_and_diffuse *= T(1) - m.transmission;
        v3 specular_bsdf = sheen_and_diffuse;
        if (m.specular > T(0))
            specular_bsdf = mx_dielectric_brdf_reflection(Lw, Vw, m.specular, m.specularColor,
                m.specularIOR, c.main_roughness, sh.normal, c.main_tangent, sheen_and_diffuse);
        v3 metalness_mix = specular_bsdf;
        if (m.metalness > T(0))
        {
            v3 refl  = m.metalColor * m.base;
            v3 edge  = m.specularColor * m.specular;
            v3 metal = mx_conductor_brdf_reflection(
                Lw, Vw, T(1), refl, edge, c.main_roughness, sh.normal, c.main_tangent);
            metalness_mix = mx_mix(specular_bsdf, metal, m.metalness);
        }
        v3 final_color = metalness_mix;
        if (m.coat > T(0))
        {
            v2 coat_roughness   = mx_roughness_anisotropy(m.coatRoughness, m.coatAnisotropy);
            v3 coat_attenuation = lerp(v3(1), m.coatColor, m.coat);
            v3 attenuated       = coat_attenuation * metalness_mix;
            final_color = mx_dielectric_brdf_reflection(Lw, Vw, m.coat, m.coatColor, m.coatIOR,
                coat_roughness, sh.normal, c.coat_tangent, attenuated);
        }
        return final_color;
    }

    // StandardSurfaceBSDF.slang:137-147
    static T calculateGGXPDF(const v3& V, v2 alpha, const v3& L)
    {
        v3 H    = normalize(V + L);
        T denom = T(4) * dot(V, H);
        return evaluateGGXSmithVNDF(V, H, alpha) / denom;
    }
    // StandardSurfaceBSDF.slang:152-174
    static v3 calculateGGXLightDirectionAndPDF(const v3& X, const v3& Y, const v3& N,
        const v3& V, v2 alpha, v2 random, v3& Lw, T& pdf)
    {
        bool flip = V.z <= T(0);
        v3 H      = sampleGGXSmithVNDF(flip ? -V : V, alpha, random);
        H         = flip ? -H : H;
        v3 L      = reflect(-V, H);
        T denom   = T(4) * dot(V, H);
        pdf       = evaluateGGXSmithVNDF(V, H, alpha) / denom;
        Lw        = tangentToWorld(L, X, Y, N);
        return L;
    }
    // StandardSurfaceBSDF.slang:122-129
    static v3 calculateHemisphereLightDirection(const v3& V, v2 random, T& pdf)
    {
        v3 Nh(0, 0, V.z > T(0) ? T(1) : T(-1));
        return sampleHemisphere(random, Nh, pdf);
    }

    // StandardSurfaceBSDF.slang:862-1088
    static v3 evaluateMaterialAndPDF(const Material<T>& m, const ShadingData<T>& sh,
        const v3& Vw, const v3& Lw, v2 random, T& pdf, int& lobeID)
    {
        v3 N = sh.normal, X = sh.tangent, Y = sh.bitangent;
        v3 V    = worldToTangent(Vw, X, Y, N);
        v3 L    = worldToTangent(Lw, X, Y, N);
        T NdotV = std::fabs(V.z);
        pdf     = T(0);
        lobeID  = NO_SECONDARY_RAY;
        Common c = prepare(m, sh);
        v3 result;
        T coat          = m.coat;
        T coatF0        = mx_ior_to_f0(m.coatIOR);
        v3 coatF        = v3(mx_fresnel_schlick(NdotV, coatF0));
        T coatLuminance = luminance(coatF * coat * m.coatColor);
        if (random.x < coatLuminance)
        {
            random.x        = remapPass(random.x, coatLuminance);
            v2 coatAlpha    = mx_roughness_anisotropy(m.coatRoughness, m.coatAnisotropy);
            pdf             = calculateGGXPDF(V, coatAlpha, L);
            v2 coatRough    = mx_roughness_anisotropy(m.coatRoughness, m.coatAnisotropy);
            result = mx_dielectric_brdf_specular_layer(
                Lw, Vw, m.coatColor * m.coat, m.coatIOR, coatRough, N, c.coat_tangent);
            lobeID = COAT_LOBE;
        }
        else
        {
            random.x     = remapFail(random.x, coatLuminance);
            v2 specAlpha = mx_roughness_anisotropy(m.specularRoughness, m.specularAnisotropy);
            if (random.x < m.metalness)
            {
                random.x = remapPass(random.x, m.metalness);
                pdf      = calculateGGXPDF(V, specAlpha, L);
                v3 refl  = m.metalColor * m.base;
                v3 edge  = m.specularColor * m.specular;
                result   = mx_conductor_brdf_reflection(
                    Lw, Vw, T(1), refl, edge, c.main_roughness, N, c.main_tangent);
                result /= std::fabs(L.z);
                lobeID = METAL_LOBE;
            }
            else
            {
                random.x        = remapFail(random.x, m.metalness);
                T F0            = mx_ior_to_f0(m.specularIOR);
                v3 F            = v3(mx_fresnel_schlick(NdotV, F0));
                T specLuminance = luminance(F * m.specular * m.specularColor);
                T glossyProb    = specLuminance;
                if (random.x < glossyProb)
                {
                    random.x = remapPass(random.x, glossyProb);
                    pdf      = calculateGGXPDF(V, specAlpha, L);
                    result   = mx_dielectric_brdf_specular_layer(Lw, Vw,
                        m.specularColor * m.specular, m.specularIOR, c.main_roughness, sh.normal,
                        c.main_tangent);
                    result /= glossyProb;
                    lobeID = GLOSSY_LOBE;
                }
                else
                {
                    random.x     = remapFail(random.x, glossyProb);
                    T sheenAlpha = clampT(m.sheenRoughness, EPS, T(1));
                    T sheen      = m.sheen;
                    if (random.x < m.sheen)
                    {
                        random.x = remapPass(random.x, sheen);
                        pdf      = divPi(dot(N, Lw));
                        v3 H     = normalize(L + V);
                        result   = mx_sheen_brdf_specular_layer(
                            Lw, Vw, m.sheen, m.sheenColor, m.sheenRoughness, N);
                        pdf    = mx_imageworks_sheen_NDF(H.z, sheenAlpha);
                        lobeID = SHEEN_LOBE;
                    }
                    else
                    {
                        random.x = remapFail(random.x, sheen);
                        pdf      = divPi(dot(N, Lw));
                        result   = mx_dielectric_brdf_diffuse_layer(Lw, Vw, m.base, m.specularIOR,
                            c.main_roughness, N, c.coat_affected_diffuse_color);
                        T dirAlbedo = mx_imageworks_sheen_directional_albedo(NdotV, sheenAlpha);
                        result *= (T(1) - dirAlbedo * m.sheen);
                        lobeID = DIFFUSE_LOBE;
                    }
                    result *= T(1); // getNonGlossyLobeCompensation: exactly 1 off the AOV path
                }
            }
            v3 coat_attenuation = lerp(v3(1), m.coatColor, m.coat);
            result *= coat_attenuation;
        }
        T NdotL = std::fabs(L.z);
        return result * NdotL;
    }

    // StandardSurfaceBSDF.slang:1093-1372
    static v3 sampleMaterial(const Material<T>& m, const ShadingData<T>& sh, const v3& Vw,
        v2 random, v3& Lw, T& pdf, int& lobeID)
    {
        v3 L;
        v3 N = sh.normal, X = sh.tangent, Y = sh.bitangent;
        v3 V    = worldToTangent(Vw, X, Y, N);
        T NdotV = std::fabs(V.z);
        Lw      = v3(1, 0, 0);
        pdf     = T(0);
        lobeID  = NO_SECONDARY_RAY;
        Common c = prepare(m, sh);
        v3 result;
        T coat          = m.coat;
        T coatF0        = mx_ior_to_f0(m.coatIOR);
        v3 coatF        = v3(mx_fresnel_schlick(NdotV, coatF0));
        T coatLuminance = luminance(coatF * coat * m.coatColor);
        if (random.x < coatLuminance)
        {
            random.x     = remapPass(random.x, coatLuminance);
            v2 coatAlpha = mx_roughness_anisotropy(m.coatRoughness, m.coatAnisotropy);
            L = calculateGGXLightDirectionAndPDF(X, Y, N, V, coatAlpha, random, Lw, pdf);
            v2 coatRough = mx_roughness_anisotropy(m.coatRoughness, m.coatAnisotropy);
            result       = mx_dielectric_brdf_specular_layer(
                Lw, Vw, m.coatColor * coat, m.coatIOR, coatRough, N, c.coat_tangent);
            result /= coatLuminance;
            lobeID = COAT_LOBE;
        }
        else
        {
            random.x     = remapFail(random.x, coatLuminance);
            v2 specAlpha = mx_roughness_anisotropy(m.specularRoughness, m.specularAnisotropy);
            if (random.x < m.metalness)
            {
                random.x = remapPass(random.x, m.metalness);
                L = calculateGGXLightDirectionAndPDF(X, Y, N, V, specAlpha, random, Lw, pdf);
                v3 refl = m.metalColor * m.base;
                v3 edge = m.specularColor * m.specular;
                result  = mx_conductor_brdf_reflection(
                    Lw, Vw, T(1), refl, edge, c.main_roughness, N, c.main_tangent);
                result /= std::fabs(L.z);
                lobeID = METAL_LOBE;
            }
            else
            {
                random.x        = remapFail(random.x, m.metalness);
                T F0            = mx_ior_to_f0(m.specularIOR);
                v3 F            = v3(mx_fresnel_schlick(NdotV, F0));
                T specLuminance = luminance(F * m.specular * m.specularColor);
                T glossyProb    = specLuminance;
                if (random.x < glossyProb)
                {
                    random.x = remapPass(random.x, glossyProb);
                    L = calculateGGXLightDirectionAndPDF(X, Y, N, V, specAlpha, random, Lw, pdf);
                    result = mx_dielectric_brdf_specular_layer(Lw, Vw,
                        m.specularColor * m.specular, m.specularIOR, c.main_roughness, sh.normal,
                        c.main_tangent);
                    result /= glossyProb;
                    lobeID = GLOSSY_LOBE;
                }
                else
                {
                    random.x     = remapFail(random.x, glossyProb);
                    T sheenAlpha = clampT(m.sheenRoughness, EPS, T(1));
                    T sheen      = m.sheen;
                    if (random.x < m.sheen)
                    {
                        random.x = remapPass(random.x, sheen);
                        L        = calculateHemisphereLightDirection(V, random, pdf);
                        Lw       = tangentToWorld(L, X, Y, N);
                        v3 H     = normalize(L + V);
                        result   = mx_sheen_brdf_specular_layer(
                            Lw, Vw, m.sheen, m.sheenColor, m.sheenRoughness, N);
                        pdf    = mx_imageworks_sheen_NDF(H.z, sheenAlpha);
                        lobeID = SHEEN_LOBE;
                    }
                    else
                    {
                        random.x       = remapFail(random.x, sheen);
                        T transmission = m.transmission;
                        if (random.x < transmission)
                        {
                            random.x       = remapPass(random.x, transmission);
                            bool reflected = false;
                            L              = -V;
                            if (!m.thinWalled)
                                L = computeRefraction(V, m.specularIOR, reflected);
                            Lw     = tangentToWorld(L, X, Y, N);
                            result = m.transmissionColor;
                            result /= std::fabs(L.z);
                            pdf    = T(1);
                            lobeID = reflected ? GLOSSY_LOBE : TRANSMISSION_LOBE;
                        }
                        else
                        {
                            random.x = remapFail(random.x, transmission);
                            L        = calculateHemisphereLightDirection(V, random, pdf);
                            Lw       = tangentToWorld(L, X, Y, N);
                            result   = mx_dielectric_brdf_diffuse_layer(Lw, Vw, m.base,
                                m.specularIOR, c.main_roughness, N, c.coat_affected_diffuse_color);
                            T dirAlbedo = mx_imageworks_sheen_directional_albedo(NdotV, sheenAlpha);
                            result *= (T(1) - dirAlbedo * m.sheen);
                            lobeID = DIFFUSE_LOBE;
                        }
                    }
                    result *= T(1); // getNonGlossyLobeCompensation: exactly 1 off the AOV path
                }
            }
            v3 coat_attenuation = lerp(v3(1), m.coatColor, m.coat);
            result *= coat_attenuation;
        }
        T NdotL = std::fabs(L.z);
        return result * NdotL;
    }
};

} // namespace orc
