// Oracle (test infrastructure, never linked into the product): plain-data layouts of the scene the
// CPU restatement renders.  Each struct mirrors a reference layout byte for byte so the same bytes
// can be handed to the oracle and to the CUDA product through their C ABIs:
//   MaterialBlock  <- Shaders/DefaultMaterialUniformBuffer.slang (400-byte std140 block, property
//                     order from MaterialBase.cpp:28-86)
//   FrameData      <- RendererBase.h:136-241 (FrameData) with SceneBase.h:34-59 (LightData)
//   EnvData        <- EnvironmentBase.h:33-55 (EnvironmentData)
//   AliasEntry     <- AliasMap.h:23-29 (Entry)
#pragma once

#include <cstddef>
#include <cstdint>

#include "../include/agb.h" // agb_graph_op and its operation / input / output codes

namespace orc
{

struct MaterialBlock
{
    float base;
    float baseColor[3];
    float diffuseRoughness;
    float metalness;
    float specular;
    int32_t _pad0;
    float specularColor[3];
    float specularRoughness;
    float specularIOR;
    float specularAnisotropy;
    float specularRotation;
    float transmission;
    float transmissionColor[3];
    float subsurface;
    float subsurfaceColor[3];
    int32_t _pad1;
    float subsurfaceRadius[3];
    float subsurfaceScale;
    float subsurfaceAnisotropy;
    float sheen;
    int32_t _pad2;
    int32_t _pad3;
    float sheenColor[3];
    float sheenRoughness;
    float coat;
    float coatColor[3];
    float coatRoughness;
    float coatAnisotropy;
    float coatRotation;
    float coatIOR;
    float coatAffectColor;
    float coatAffectRoughness;
    float emission;
    int32_t _pad4;
    float emissionColor[3];
    int32_t _pad5;
    float opacity[3];
    int32_t thinWalled;
    // Five texture slots, each {has, offset, (pad), scale, pivot, rotation}.
    int32_t hasBaseColorTex;
    float baseColorTexOffset[2];
    int32_t _pad6;
    float baseColorTexScale[2];
    float baseColorTexPivot[2];
    float baseColorTexRotation;
    int32_t hasSpecularRoughnessTex;
    float specularRoughnessTexOffset[2];
    float specularRoughnessTexScale[2];
    float specularRoughnessTexPivot[2];
    float specularRoughnessTexRotation;
    int32_t hasEmissionColorTex;
    float emissionColorTexOffset[2];
    float emissionColorTexScale[2];
    float emissionColorTexPivot[2];
    float emissionColorTexRotation;
    int32_t hasOpacityTex;
    float opacityTexOffset[2];
    float opacityTexScale[2];
    float opacityTexPivot[2];
    float opacityTexRotation;
    int32_t hasNormalTex;
    float normalTexOffset[2];
    float normalTexScale[2];
    float normalTexPivot[2];
    float normalTexRotation;
    int32_t _pad7;
    int32_t _pad8;
    int32_t _pad9;
};
static_assert(sizeof(MaterialBlock) == 400, "Standard Surface block is 400 bytes");
static_assert(offsetof(MaterialBlock, specularColor) == 32, "layout");
static_assert(offsetof(MaterialBlock, sheenColor) == 128, "layout");
static_assert(offsetof(MaterialBlock, opacity) == 208, "layout");
static_assert(offsetof(MaterialBlock, baseColorTexScale) == 240, "layout");
static_assert(offsetof(MaterialBlock, normalTexRotation) == 384, "layout");

// Texture slots of the built-in material, in the reference order (MaterialBase.cpp:97-103).
enum TextureSlot
{
    kTexBaseColor         = 0,
    kTexSpecularRoughness = 1,
    kTexOpacity           = 2,
    kTexNormal            = 3,
    kTexEmission          = 4,
    kTexSlotCount         = 5
};

struct DistantLight
{
    float colorAndIntensity[4];
    float direction[3]; // already negated: points toward the light
    float cosRadius;
};

struct LightData
{
    DistantLight distantLights[4];
    int32_t distantLightCount;
    int32_t pad[3];
};
static_assert(sizeof(LightData) == 144, "LightData layout");

struct FrameData
{
    float cameraViewProj[16];
    float cameraViewProjPrev[16];
    // Camera-to-world matrix stored row-major: right=(m0,m4,m8) up=(m1,m5,m9) back=(m2,m6,m10)
    // eye=(m3,m7,m11).  These are the bytes of the reference's transpose(inverse(view)).
    float cameraInvView[16];
    float cameraInvViewPrev[16];
    float viewSize[2];
    float cameraJitter[2];
    float cameraJitterPrev[2];
    int32_t isOrthoProjection;
    float focalDistance;
    float lensRadius;
    float timeDeltaMs;
    int32_t isTemporalJitterEnabled;
    float sceneSize;
    int32_t isForceOpaqueShadowsEnabled;
    int32_t isDepthNDCEnabled;
    int32_t isDiffuseOnlyEnabled;
    int32_t isDisplayErrorsEnabled;
    int32_t isDenoisingEnabled;
    int32_t isDenoisingAOVsEnabled;
    int32_t traceDepth;
    float maxLuminance;
    int32_t isRussianRouletteEnabled;
    int32_t russianRouletteStartDepth;
    int32_t isPathRegularizationEnabled;
    float pathRegularizationStrength;
    float indirectBounceClampScale;
    float skyViewZ;
    float _padding1[2];
    LightData lights;
};
static_assert(offsetof(FrameData, viewSize) == 256, "FrameData layout");
static_assert(offsetof(FrameData, traceDepth) == 328, "FrameData layout");
static_assert(offsetof(FrameData, lights) == 368, "FrameData layout");
static_assert(sizeof(FrameData) == 512, "FrameData layout");

struct EnvData
{
    float lightTop[3];
    float _padding1;
    float lightBottom[3];
    float lightTexLuminanceIntegral;
    // 4x4 matrices stored row-major; applied to column vectors.
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
static_assert(sizeof(EnvData) == 268, "EnvData layout");

struct AliasEntry
{
    uint32_t alias;
    float prob;
    float pdf;
    float _padding1;
};
static_assert(sizeof(AliasEntry) == 16, "AliasEntry layout");

// An RGBA32F image (material texture or environment).  Sampled with repeat addressing; `linear`
// selects bilinear filtering, otherwise nearest.
struct Image
{
    const float* rgba = nullptr; // width*height*4 floats, row 0 at the top (v = 0)
    uint32_t width    = 0;
    uint32_t height   = 0;
    int32_t linear    = 0;
};

// A triangle mesh in object space.  Normals and UVs are optional (null).
struct Mesh
{
    const float* positions = nullptr; // 3 floats per vertex
    const float* normals   = nullptr; // 3 floats per vertex or null
    const float* texcoords = nullptr; // 2 floats per vertex or null
    const uint32_t* indices = nullptr; // 3 per triangle
    uint32_t vertexCount   = 0;
    uint32_t triangleCount = 0;
};

// One material layer on an instance (the DirectX layer data, GlobalBufferAccessors.slang:60-83):
// a material and a per-vertex UV set of the base mesh's vertex count.
struct Layer
{
    int32_t material = 0;
    const float* texcoords = nullptr; // 2 floats per base-mesh vertex
};

struct Instance
{
    int32_t mesh     = 0;
    int32_t material = 0;
    float objectToWorld[12]; // 3x4 row-major
    int32_t layerCount = 0;
    const Layer* layers = nullptr;
};

// Per-material texture bindings, one image index per TextureSlot (-1 = none).
struct MaterialTextures
{
    int32_t image[kTexSlotCount];
};

} // namespace orc
