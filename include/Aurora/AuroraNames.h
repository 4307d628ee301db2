// Property, attribute and type names of Aurora's public interface (Libraries/Aurora/API/Aurora/
// AuroraNames.h), declared as in that header so that clients compiled against either link
// against this backend; the backend defines them (aurora_gb300/csrc/agb_aurora_api.cpp) with the
// values of Libraries/Aurora/Source/AuroraNames.cpp.
#pragma once

namespace Aurora
{
namespace Names
{

struct InstanceProperties
{
    static AURORA_API const std::string kGeometry;
    static AURORA_API const std::string kMaterial;
    static AURORA_API const std::string kTransform;
    static AURORA_API const std::string kObjectID;
    static AURORA_API const std::string kVisible;
    static AURORA_API const std::string kSelectable;
    static AURORA_API const std::string kMaterialLayers; // innermost layer first
    static AURORA_API const std::string kGeometryLayers;
};

struct EnvironmentProperties
{
    static AURORA_API const std::string kLightTop;
    static AURORA_API const std::string kLightBottom;
    static AURORA_API const std::string kLightImage;
    static AURORA_API const std::string kLightTransform;
    static AURORA_API const std::string kBackgroundTop;
    static AURORA_API const std::string kBackgroundBottom;
    static AURORA_API const std::string kBackgroundImage;
    static AURORA_API const std::string kBackgroundTransform;
    static AURORA_API const std::string kBackgroundUseScreen;
};

struct AddressModes
{
    static AURORA_API const std::string kWrap;
    static AURORA_API const std::string kMirror;
    static AURORA_API const std::string kClamp;
    static AURORA_API const std::string kBorder;
    static AURORA_API const std::string kMirrorOnce;
};

struct SamplerProperties
{
    static AURORA_API const std::string kAddressModeU;
    static AURORA_API const std::string kAddressModeV;
};

struct VertexAttributes
{
    static AURORA_API const std::string kPosition;
    static AURORA_API const std::string kNormal;
    static AURORA_API const std::string kTangent;
    static AURORA_API const std::string kTexCoord0;
    static AURORA_API const std::string kTexCoord1;
    static AURORA_API const std::string kTexCoord2;
    static AURORA_API const std::string kTexCoord3;
    static AURORA_API const std::string kTexCoord4;
    static AURORA_API const std::string kIndices;
};

struct MaterialTypes
{
    static AURORA_API const std::string kBuiltIn;
    static AURORA_API const std::string kMaterialX;
    static AURORA_API const std::string kMaterialXPath;
};

struct UpscalerModes
{
    static AURORA_API const std::string kNone;
    static AURORA_API const std::string kDLSS;
    static AURORA_API const std::string kFSR;
    static AURORA_API const std::string kDLSSRayReconstruction;
};

struct LightTypes
{
    static AURORA_API const std::string kDistantLight;
};

struct LightProperties
{
    static AURORA_API const std::string kDirection;
    static AURORA_API const std::string kAngularDiameter;
    static AURORA_API const std::string kExposure;
    static AURORA_API const std::string kIntensity;
    static AURORA_API const std::string kColor;
};

} // namespace Names
} // namespace Aurora
