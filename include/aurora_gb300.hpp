// aurora_gb300.hpp - C++ renderer interface of the GB300 backend, mirroring the part of Aurora's
// public API (Libraries/Aurora/API/Aurora/Aurora.h) that the path-tracing hot path uses: the same
// class and method names, argument meanings, property names (AuroraNames.cpp) and renderer option
// names (RendererBase.cpp:59-89), implemented over the C ABI in agb.h.  Code written against
// Aurora's IRenderer / IScene / IRenderBuffer for this path builds against this header by
// changing the namespace.
//
// Differences from Aurora, by design:
//   * matrices are std::array<float, 16> in glm's column-major memory order (element (row r,
//     column c) at 4 * c + r) and vectors std::array<float, 3>;
//   * only the built-in Standard Surface material type, triangle geometry, distant lights and
//     lat-long environment images (Float_RGB / Float_RGBA / Integer_RGBA) are supported;
//   * shadows are always opaque (the HGI backend's setting, HGIRenderer.cpp:491);
//   * errors Aurora reports with AU_FAIL throw agb_aurora::Error; those it reports with AU_ERROR
//     go to the log callback (stderr by default).
#pragma once

#include <array>
#include <cstdint>
#include <functional>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <variant>
#include <vector>

#if defined(_WIN32)
#define AGB_CPP_API __declspec(dllexport)
#else
#define AGB_CPP_API __attribute__((visibility("default")))
#endif

namespace agb_aurora
{

using Path  = std::string;
using Paths = std::vector<Path>;
using vec2  = std::array<float, 2>;
using vec3  = std::array<float, 3>;
using mat4  = std::array<float, 16>;
using Strings = std::vector<std::string>;

struct Error : std::runtime_error
{
    using std::runtime_error::runtime_error;
};
// Receives recoverable errors (Aurora's AU_ERROR); null restores the stderr default.
AGB_CPP_API void setLogCallback(std::function<void(const std::string&)> cb);

// A property value (Aurora.h:125-300, reduced to the kinds this path uses).  std::monostate is
// Aurora's undefined value: set through a property map it returns the property to its default
// (ResourceStub.cpp:278-292, RendererBase.cpp:166-168).
using PropertyValue = std::variant<bool, int, float, vec2, vec3, mat4, std::string, Strings, std::monostate>;
using Properties    = std::map<std::string, PropertyValue>;

// Property names (AuroraNames.cpp).
namespace Names
{
namespace InstanceProperties
{
inline const std::string kMaterial("material");
inline const std::string kTransform("transform");
inline const std::string kVisible("visible");
inline const std::string kMaterialLayers("layer_materials");
inline const std::string kGeometryLayers("layer_geometry");
} // namespace InstanceProperties
namespace EnvironmentProperties
{
inline const std::string kLightTop("light_top");
inline const std::string kLightBottom("light_bottom");
inline const std::string kLightImage("light_image");
inline const std::string kLightTransform("light_transform");
inline const std::string kBackgroundTop("background_top");
inline const std::string kBackgroundBottom("background_bottom");
inline const std::string kBackgroundImage("background_image");
inline const std::string kBackgroundTransform("background_transform");
inline const std::string kBackgroundUseScreen("background_use_screen");
} // namespace EnvironmentProperties
namespace VertexAttributes
{
inline const std::string kPosition("position");
inline const std::string kNormal("normal");
inline const std::string kTexCoord0("tcoord0");
inline const std::string kIndices("indices");
} // namespace VertexAttributes
namespace SamplerProperties
{
inline const std::string kAddressModeU("AddressModeU");
inline const std::string kAddressModeV("AddressModeV");
} // namespace SamplerProperties
namespace AddressModes
{
inline const std::string kWrap("Wrap");
inline const std::string kMirror("Mirror");
inline const std::string kClamp("Clamp");
inline const std::string kBorder("Border");
inline const std::string kMirrorOnce("MirrorOnce");
} // namespace AddressModes
namespace LightTypes
{
inline const std::string kDistantLight("DistantLight");
} // namespace LightTypes
namespace LightProperties
{
inline const std::string kDirection("direction");
inline const std::string kAngularDiameter("angular_diameter_radians");
inline const std::string kIntensity("intensity");
inline const std::string kColor("color");
} // namespace LightProperties
namespace MaterialTypes
{
inline const std::string kBuiltIn("BuiltIn");
// A MaterialX document (the string) or the path of a .mtlx file (AuroraNames.cpp:48-50): a
// standard_surface with constant inputs, read into the built-in material's properties.
inline const std::string kMaterialX("MaterialX");
inline const std::string kMaterialXPath("MaterialXPath");
} // namespace MaterialTypes
} // namespace Names

enum class ImageFormat
{
    Integer_RGBA,
    Float_RGBA,
    Float_RGB
};
enum class AttributeFormat
{
    Float3,
    Float2,
    UInt
};
enum class PrimitiveType
{
    Triangles
};

// Geometry pulled by the renderer when an instance first needs it (Aurora.h:470-525).
struct AttributeData
{
    const void* address = nullptr;
    size_t size         = 0;
    size_t offset       = 0;
    size_t stride       = 0;
};
using AttributeDataMap = std::map<std::string, AttributeData>;
using GetAttributeDataFunction = std::function<bool(AttributeDataMap& buffers, size_t firstVertex,
    size_t vertexCount, size_t firstIndex, size_t indexCount)>;
using AttributeUpdateCompleteFunction = std::function<void(const AttributeDataMap& buffers,
    size_t firstVertex, size_t vertexCount, size_t firstIndex, size_t indexCount)>;
struct VertexDescription
{
    std::map<std::string, AttributeFormat> attributes;
    size_t count = 0;
};
struct GeometryDescriptor
{
    PrimitiveType type = PrimitiveType::Triangles;
    VertexDescription vertexDesc;
    size_t indexCount = 0;
    GetAttributeDataFunction getAttributeData               = nullptr;
    AttributeUpdateCompleteFunction attributeUpdateComplete = nullptr;
};

// Images, pulled the same way (Aurora.h:528-600).
struct ImageData
{
    const void* pPixelBuffer  = nullptr;
    size_t bytesPerRow        = 0;
    size_t bufferSize         = 0;
    std::array<int, 2> dimensions = { 0, 0 };
    ImageFormat format        = ImageFormat::Integer_RGBA;
    bool overrideLinearize    = false; // use `linearize` below instead of the descriptor's
    bool linearize            = true;
};
struct ImageDescriptor
{
    bool linearize = true;
    std::function<bool(ImageData& data)> getData          = nullptr;
    std::function<void(const ImageData& data)> updateComplete = nullptr;
};

class IValues
{
public:
    virtual void setBoolean(const std::string& name, bool value)             = 0;
    virtual void setInt(const std::string& name, int value)                  = 0;
    virtual void setFloat(const std::string& name, float value)              = 0;
    virtual void setFloat3(const std::string& name, const vec3& value)       = 0;
    virtual void setMatrix(const std::string& name, const mat4& value)       = 0;
    virtual void setString(const std::string& name, const std::string& value) = 0;
    virtual void clearValue(const std::string& name)                         = 0;
    virtual ~IValues() = default;
};

class ILight
{
public:
    virtual IValues& values() = 0;
    virtual ~ILight()        = default;
};
using ILightPtr = std::shared_ptr<ILight>;

// Ground plane (Aurora.h:780-806): values "enabled" (bool), "position", "normal" (float3),
// "shadow_opacity", "reflection_opacity", "reflection_roughness" (float), "shadow_color",
// "reflection_color" (float3); defaults as PTGroundPlane.cpp:42-51.
class IGroundPlane
{
public:
    virtual IValues& values()   = 0;
    virtual ~IGroundPlane()     = default;
};
using IGroundPlanePtr = std::shared_ptr<IGroundPlane>;

// A render target (Aurora.h:714-747): RGBA8 (Integer_RGBA) or RGBA32F (Float_RGBA).
class IRenderBuffer
{
public:
    // A readable (or shareable) buffer held for as long as the pointer lives (Aurora.h:720-733).
    class IBuffer
    {
    public:
        virtual const void* data() = 0;
        virtual const void* handle() { return nullptr; }
        virtual ~IBuffer() = default;
    };
    using IBufferPtr = std::shared_ptr<IBuffer>;
    // The pixels of the last render; stride receives the bytes per row.
    virtual const void* data(size_t& stride, bool removePadding = false) = 0;
    // The pixels of the last render in a buffer of their own (a copy: later renders leave it).
    virtual IBufferPtr asReadable(size_t& stride) = 0;
    // Shareable GPU memory of the target: none here (post-processing writes host memory), null.
    virtual IBufferPtr asShared() = 0;
    virtual int width() const                                           = 0;
    virtual int height() const                                          = 0;
    virtual ~IRenderBuffer() = default;
};
using IRenderBufferPtr = std::shared_ptr<IRenderBuffer>;

// Scene description keyed by paths (Aurora.h:892-1041, SceneBase.h:26-163).
class IScene
{
public:
    virtual void setGeometryDescriptor(const Path& atPath, const GeometryDescriptor& desc) = 0;
    virtual void setImageDescriptor(const Path& atPath, const ImageDescriptor& desc)       = 0;
    // An image read from a file when first used (Aurora.h:905-914): PNG (8 or 16 bits, grey,
    // grey + alpha, RGB, RGBA or palette, non-interlaced) or Radiance HDR; an empty filePath
    // reads atPath.  linearize: 8-bit texels are sRGB encoded.
    virtual void setImageFromFilePath(const Path& atPath, const std::string& filePath = "",
        bool linearize = true, bool isEnvironment = false)                                = 0;
    virtual void setMaterialType(const Path& atPath,
        const std::string& materialType = Names::MaterialTypes::kBuiltIn,
        const std::string& document     = "Default")                                      = 0;
    // Material properties are the Standard Surface names (MaterialBase.cpp), with textures as
    // image paths: base_color_image, specular_roughness_image, opacity_image, normal_image,
    // emission_color_image, each with <name>_offset / _scale / _pivot (vec2), _rotation (float)
    // and _sampler (a sampler path).
    virtual void setMaterialProperties(const Path& path, const Properties& materialProperties) = 0;
    // Samplers (Aurora.h:922): AddressModeU / AddressModeV.  A texture without a sampler uses the
    // renderer's default one (nearest filtering, wrap); a texture with a sampler set here filters
    // bilinearly (HGISampler.cpp:21-41).  Address modes other than Wrap are reported and sampled
    // with wrapping.
    virtual void setSamplerProperties(const Path& atPath, const Properties& props)      = 0;
    virtual bool addInstance(const Path& path, const Path& geometry, const Properties& properties = {}) = 0;
    virtual void setInstanceProperties(const Path& path, const Properties& instanceProperties) = 0;
    virtual void removeInstance(const Path& path)                                         = 0;
    virtual bool setEnvironmentProperties(const Path& environment, const Properties& props) = 0;
    virtual bool setEnvironment(const Path& environment)                                  = 0;
    virtual void setBounds(const vec3& min, const vec3& max)                              = 0;
    virtual ILightPtr addLightPointer(const std::string& lightType)                       = 0;
    // Null restores the renderer's default ground plane, which is disabled (PTScene.cpp:660-667).
    virtual void setGroundPlanePointer(const IGroundPlanePtr& pGroundPlane)               = 0;
    virtual ~IScene() = default;
};
using IScenePtr = std::shared_ptr<IScene>;

enum class AOV
{
    Final
};
using TargetAssignments = std::map<AOV, IRenderBufferPtr>;

// Loads the bytes of a resource named by a URI (Aurora.h:54-63): the image files of
// setImageFromFilePath and of MaterialX documents.  pFileNameOut receives a file name whose
// extension selects the decoder (".hdr": Radiance RGBE; otherwise PNG).
using LoadResourceFunction =
    std::function<bool(const std::string& uri, std::vector<unsigned char>* pBufferOut, std::string* pFileNameOut)>;

// The renderer (Aurora.h:1098-1222).
class IRenderer
{
public:
    enum class Backend
    {
        Default,
        CUDA
    };
    virtual IScenePtr createScene()                                                   = 0;
    virtual IGroundPlanePtr createGroundPlanePointer()                                = 0;
    virtual void setScene(const IScenePtr& pScene)                                    = 0;
    virtual IRenderBufferPtr createRenderBuffer(int width, int height, ImageFormat format) = 0;
    virtual void setTargets(const TargetAssignments& targetAssignments)               = 0;
    virtual void setOptions(const Properties& options)                                = 0;
    virtual IValues& options()                                                        = 0;
    virtual void setCamera(const mat4& view, const mat4& proj, float focalDistance = 1.0f,
        float lensRadius = 0.0f)                                                      = 0;
    virtual void render(uint32_t sampleStart = 0, uint32_t sampleCount = 1)           = 0;
    virtual void waitForTask()                                                        = 0;
    // Built-in material types beyond the default Standard Surface: none, as in the HGI
    // backend (HGIRenderer.cpp:622-627).
    virtual const std::vector<std::string>& builtInMaterials()                       = 0;
    // The loader for image files named by path (Aurora.h:1206-1208); without one (or after an
    // empty function) files are read from the file system.  Scenes created before the call use it
    // too.
    virtual void setLoadResourceFunction(LoadResourceFunction func)                  = 0;
    virtual ~IRenderer() = default;
};
using IRendererPtr = std::shared_ptr<IRenderer>;

// Aurora::createRenderer (Aurora.cpp:31-69): null when no sm_103a device can be used.
AGB_CPP_API IRendererPtr createRenderer(IRenderer::Backend backend = IRenderer::Backend::Default,
    uint32_t taskCount = 3);

} // namespace agb_aurora
