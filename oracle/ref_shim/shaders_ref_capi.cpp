// C entry points over the reference's own shader functions, compiled as host C++ (test
// infrastructure: the pin of the oracle and of the device kernels; never part of the product).
//
// oracle/build_oracle.py generates oracle/_ref/gen/*.slang.h from the reference's unmodified
// Shaders/{Globals,Colors,Random,Sampling,BSDFCommon,Material,StandardSurfaceBSDF,Environment}.slang
// by a mechanical rewrite, and compiles this file twice: REF_PREC 32 (the shaders' own FP32
// arithmetic, exported as ref32_*) and REF_PREC 64 (the same source with `float` as double,
// exported as ref64_*).
//
// Inputs follow the oracle's batch conventions (oracle/oracle_capi.cpp): 400-byte Standard Surface
// blocks (Shaders/DefaultMaterialUniformBuffer.slang) mapped to the shaders' Material the way
// evaluateDefaultMaterial does (DefaultMaterial.slang:130-239, no textures; metal colour = base
// colour), shading frames of 12 floats (normal, tangent, bitangent, unused).
#include <cstddef>
#include <cstdint>

#if REF_PREC == 64
#define REF_REAL double
#define REF_EXPORT(name) ref64_##name
#else
#define REF_REAL float
#define REF_EXPORT(name) ref32_##name
#endif

#include "hlsl.h"
#include "pipeline_state.h"

#if REF_PREC == 64
// The generated shader code names its scalar type `float`; here it computes in double.  Float
// literals (HLSL's type for an unsuffixed literal) keep their FP32 values.
#define float double
#endif

// Inside namespace hlsl, so the intrinsics there take precedence over the C library's; internal
// linkage, as the two precisions' copies of the same functions live in one library.
namespace hlsl
{
namespace
{
#include "Colors.slang.h"
#include "Random.slang.h"
#include "Material.slang.h"
#include "StandardSurfaceBSDF.slang.h"
#include "Environment.slang.h"
} // namespace
} // namespace hlsl

#if REF_PREC == 64
#undef float
#endif

#define REF_API extern "C" __attribute__((visibility("default")))

namespace
{

// Offsets of the 400-byte block (DefaultMaterialUniformBuffer.slang).
struct Block
{
    const uint8_t* p;
    float f(size_t off) const
    {
        float v;
        std::memcpy(&v, p + off, 4);
        return v;
    }
    float3 f3(size_t off) const { return float3(f(off), f(off + 4), f(off + 8)); }
    int i(size_t off) const
    {
        int v;
        std::memcpy(&v, p + off, 4);
        return v;
    }
};

Material materialFromBlock(const uint8_t* block)
{
    Block b{ block };
    Material m;
    m.base                 = b.f(0);
    m.baseColor            = b.f3(4);
    m.diffuseRoughness     = b.f(16);
    m.metalness            = b.f(20);
    m.specular             = b.f(24);
    m.specularColor        = b.f3(32);
    m.specularRoughness    = b.f(44);
    m.specularIOR          = b.f(48);
    m.specularAnisotropy   = b.f(52);
    m.specularRotation     = b.f(56);
    m.transmission         = b.f(60);
    m.transmissionColor    = b.f3(64);
    m.subsurface           = b.f(76);
    m.subsurfaceColor      = b.f3(80);
    m.subsurfaceRadius     = b.f3(96);
    m.subsurfaceScale      = b.f(108);
    m.subsurfaceAnisotropy = b.f(112);
    m.sheen                = b.f(116);
    m.sheenColor           = b.f3(128);
    m.sheenRoughness       = b.f(140);
    m.coat                 = b.f(144);
    m.coatColor            = b.f3(148);
    m.coatRoughness        = b.f(160);
    m.coatAnisotropy       = b.f(164);
    m.coatRotation         = b.f(168);
    m.coatIOR              = b.f(172);
    m.coatAffectColor      = b.f(176);
    m.coatAffectRoughness  = b.f(180);
    m.emission             = b.f(184);
    m.emissionColor        = b.f3(192);
    m.opacity              = b.f3(208);
    m.thinWalled           = b.i(220) != 0;
    m.isOpaque             = true;
    m.metalColor           = m.baseColor;
    return m;
}

float3 load3(const float* p) { return float3(p[0], p[1], p[2]); }

void store3(float* p, const float3& v)
{
    p[0] = static_cast<float>(v.x);
    p[1] = static_cast<float>(v.y);
    p[2] = static_cast<float>(v.z);
}

float4x4 matrixFrom(const float* m)
{
    float4x4 r;
    for (int k = 0; k < 4; k++)
        r[k] = float4(m[4 * k], m[4 * k + 1], m[4 * k + 2], m[4 * k + 3]);
    return r;
}

// EnvironmentBase::EnvironmentData as the oracle and the device store it (268 bytes).
struct EnvBlock
{
    float lightTop[3];
    float _padding1;
    float lightBottom[3];
    float lightTexLuminanceIntegral;
    float lightTransform[16];
    float lightTransformInv[16];
    float backgroundTop[3];
    float _padding3;
    float backgroundBottom[3];
    float _padding4;
    float backgroundTransform[16];
    int32_t backgroundUseScreen;
    int32_t hasLightTex;
    int32_t hasBackgroundTex;
};
static_assert(sizeof(EnvBlock) == 268, "EnvironmentData layout");

Environment environmentFrom(const EnvBlock& e, const float* light, uint32_t lw, uint32_t lh,
    const float* background, uint32_t bw, uint32_t bh, int linear, const void* alias)
{
    Environment env;
    EnvironmentConstants& c     = env.constants;
    c.lightTop                  = load3(e.lightTop);
    c.lightBottom               = load3(e.lightBottom);
    c.lightTexLuminanceIntegral = e.lightTexLuminanceIntegral;
    c.lightTransform            = matrixFrom(e.lightTransform);
    c.lightTransformInv         = matrixFrom(e.lightTransformInv);
    c.backgroundTop             = load3(e.backgroundTop);
    c.backgroundBottom          = load3(e.backgroundBottom);
    c.backgroundTransform       = matrixFrom(e.backgroundTransform);
    c.backgroundUseScreen       = e.backgroundUseScreen;
    c.hasLightTex               = e.hasLightTex;
    c.hasBackgroundTex          = e.hasBackgroundTex;
    env.lightTexture.rgba       = light;
    env.lightTexture.width      = lw;
    env.lightTexture.height     = lh;
    env.backgroundTexture.rgba  = background;
    env.backgroundTexture.width = bw;
    env.backgroundTexture.height = bh;
    env.sampler.linear          = linear;
    env.aliasMap.data           = static_cast<const AliasEntry*>(alias);
    return env;
}

} // namespace

// op 0: evaluateMaterial (StandardSurfaceBSDF.slang:598-718); op 1: sampleMaterial (:1093-1372);
// op 2: evaluateMaterialAndPDF (:862-1088).  World-space V, L; rnd pairs for ops 1 and 2.
REF_API void REF_EXPORT(bsdf_batch)(int op, int denoisingAOVs, const void* materials,
    const int32_t* matIndex, const float* frames, const float* V, const float* L, const float* rnd,
    int64_t n, float* outValue, float* outDir, float* outPdf, int32_t* outLobe)
{
    gFrameData.isDenoisingAOVsEnabled = denoisingAOVs;
    const uint8_t* blocks = static_cast<const uint8_t*>(materials);
    for (int64_t i = 0; i < n; i++)
    {
        Material m = materialFromBlock(blocks + 400 * size_t(matIndex[i]));
        ShadingData sh;
        sh.normal    = load3(frames + 12 * i);
        sh.tangent   = load3(frames + 12 * i + 3);
        sh.bitangent = load3(frames + 12 * i + 6);
        float3 v     = load3(V + 3 * i);
        float3 res(0.0f);
        if (op == 0)
            res = evaluateMaterial(m, sh, v, load3(L + 3 * i));
        else if (op == 1)
        {
            float3 lw;
            hlsl::real pdf = 0;
            int lobe = 0;
            res = sampleMaterial(m, sh, v, float2(rnd[2 * i], rnd[2 * i + 1]), lw, pdf, lobe);
            store3(outDir + 3 * i, lw);
            outPdf[i]  = static_cast<float>(pdf);
            outLobe[i] = lobe;
        }
        else
        {
            hlsl::real pdf = 0;
            int lobe = 0;
            res = evaluateMaterialAndPDF(m, sh, v, load3(L + 3 * i), float2(rnd[2 * i], rnd[2 * i + 1]),
                pdf, lobe);
            outPdf[i]  = static_cast<float>(pdf);
            outLobe[i] = lobe;
        }
        store3(outValue + 3 * i, res);
    }
    gFrameData.isDenoisingAOVsEnabled = 0;
}

// sampleEnvironment (Environment.slang:137-186) over rnd pairs.
REF_API void REF_EXPORT(env_sample)(const void* envData, const float* lightRGBA, uint32_t width,
    uint32_t height, const void* alias, const float* rnd, int64_t n, float* outRadiance,
    float* outDir, float* outPdf)
{
    const EnvBlock& e = *static_cast<const EnvBlock*>(envData);
    Environment env   = environmentFrom(e, lightRGBA, width, height, nullptr, 0, 0, 0, alias);
    for (int64_t i = 0; i < n; i++)
    {
        float3 L;
        hlsl::real pdf = 0;
        float3 r = sampleEnvironment(env, float2(rnd[2 * i], rnd[2 * i + 1]), L, pdf);
        store3(outRadiance + 3 * i, r);
        store3(outDir + 3 * i, L);
        outPdf[i] = static_cast<float>(pdf);
    }
}

// evaluateEnvironment (Environment.slang:98-133) in world directions, as light or background.
REF_API void REF_EXPORT(env_evaluate)(const void* envData, const float* lightRGBA, uint32_t lw,
    uint32_t lh, const float* backgroundRGBA, uint32_t bw, uint32_t bh, int linear,
    const float* dirs, const int32_t* asBackground, int64_t n, float* out)
{
    const EnvBlock& e = *static_cast<const EnvBlock*>(envData);
    Environment env   = environmentFrom(e, lightRGBA, lw, lh, backgroundRGBA, bw, bh, linear, nullptr);
    for (int64_t i = 0; i < n; i++)
        store3(out + 3 * i, evaluateEnvironment(env, load3(dirs + 3 * i), asBackground[i] != 0));
}

// The first n random2D pairs of pixel (px, py) for a sample index (Random.slang:96-146).
REF_API void REF_EXPORT(random_stream)(uint32_t sampleIndex, uint32_t width, uint32_t px,
    uint32_t py, int n, float* out)
{
    Random rng = initRand(sampleIndex, uint2(width, 1u), uint2(px, py));
    for (int k = 0; k < n; k++)
    {
        float2 r = random2D(rng);
        out[2 * k]     = static_cast<float>(r.x);
        out[2 * k + 1] = static_cast<float>(r.y);
    }
}
