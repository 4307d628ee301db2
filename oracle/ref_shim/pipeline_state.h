// Host stand-ins for the pipeline state the reference's shader functions read (test
// infrastructure).  The generated copy of Environment.slang includes this file in place of
// GlobalPipelineState.slang, whose resource bindings have no host meaning; the fields the
// functions read keep their names (GlobalPipelineState.slang:27-43 EnvironmentConstants,
// AliasMap.h Entry, Frame.slang isDenoisingAOVsEnabled; Geometry.slang ShadingData's frame).
#pragma once

#include "hlsl.h"

struct EnvironmentConstants
{
    float3 lightTop;
    float3 lightBottom;
    float lightTexLuminanceIntegral = 0;
    float4x4 lightTransform;
    float4x4 lightTransformInv;
    float3 backgroundTop;
    float3 backgroundBottom;
    float4x4 backgroundTransform;
    int backgroundUseScreen = 0;
    int hasLightTex         = 0;
    int hasBackgroundTex    = 0;
};

struct AliasEntry
{
    uint alias;
    float probability;
    float pdf;
    float _padding;
};

// The shading frame the BSDF functions read (Geometry.slang ShadingData: normal, tangent,
// bitangent; the rest of the structure is not read by them).
struct ShadingData
{
    float3 normal;
    float3 tangent;
    float3 bitangent;
};

struct RefFrameData
{
    int isDenoisingAOVsEnabled = 0;
};
static RefFrameData gFrameData; // one per translation unit (each precision has its own)

// Ray-dispatch indices: only the screen-space background mode reads them, which the pin does not
// exercise.
inline uint3 DispatchRaysIndex() { return uint3(0u); }
inline uint3 DispatchRaysDimensions() { return uint3(1u); }
