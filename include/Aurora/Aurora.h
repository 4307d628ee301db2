// Aurora's public C++ interface (Libraries/Aurora/API/Aurora/Aurora.h), declared for the GB300
// backend: the same namespace, classes, virtual functions in the same order, value types with the
// same members, and free functions, so that an Aurora client compiled against the reference's own
// header links against libagb_cuda.so and calls into this backend (tests/test_aurora_dropin.py
// compares the two headers' class layouts and links such a client).  The implementation over the
// C ABI is aurora_gb300/csrc/agb_aurora_api.cpp; createRenderer(Backend::Default) returns the
// CUDA path tracer.
//
// What this backend does with each call is documented beside it where it differs from the
// reference's renderers; the rest behaves as the reference's HGI backend (HGIRenderer.cpp,
// HGIScene.cpp, SceneBase.cpp).
#pragma once

#include <Aurora/Foundation/Log.h>

#include <array>
#include <cstddef>
#include <cstdint>
#include <functional>
#include <map>
#include <memory>
#include <string>
#include <string_view>
#include <unordered_map>
#include <utility>
#include <vector>

#define GLM_FORCE_CTOR_INIT
#include <glm/glm.hpp>

#if !defined(AURORA_API)
#define AURORA_API __attribute__((visibility("default")))
#endif

#include "AuroraNames.h"

#define MAKE_AURORA_PTR(_x) using _x##Ptr = std::shared_ptr<_x>

namespace Aurora
{

// Loads a resource named by a URI into a buffer: the image files named by setImageFromFilePath
// and by MaterialX documents.
using LoadResourceFunction = std::function<bool(
    const std::string& uri, std::vector<unsigned char>* pBufferOut, std::string* pFileNameOut)>;

using vec2 = glm::vec2;
using vec3 = glm::vec3;
using vec4 = glm::vec4;
using mat4 = glm::mat4;
using rgb  = glm::vec3;
using rgba = glm::vec4;

using Path     = std::string;
using PathView = std::string_view;
using Strings  = std::vector<std::string>;

// A tagged property value: the scalar and vector kinds share storage, strings keep their own.
struct PropertyValue
{
    enum class Type : uint8_t
    {
        Undefined,
        Bool,
        Int,
        Float,
        Float2,
        Float3,
        Float4,
        Matrix4,
        String,
        Strings
    };

    PropertyValue() : type(Type::Undefined) {}
    PropertyValue(const PropertyValue& in) { *this = in; }
    const PropertyValue& operator=(const PropertyValue& in)
    {
        type = in.type;
        if (type == Type::Bool)
            _bool = in._bool;
        else if (type == Type::Int)
            _int = in._int;
        else if (type == Type::Float)
            _float = in._float;
        else if (type == Type::Float2)
            _float2 = in._float2;
        else if (type == Type::Float3)
            _float3 = in._float3;
        else if (type == Type::Float4)
            _float4 = in._float4;
        else if (type == Type::Matrix4)
            _matrix4 = in._matrix4;
        else if (type == Type::String)
            _string = in._string;
        else if (type == Type::Strings)
            _strings = in._strings;
        return *this;
    }
    PropertyValue(bool v) : type(Type::Bool), _bool(v) {}
    PropertyValue(int v) : type(Type::Int), _int(v) {}
    PropertyValue(float v) : type(Type::Float), _float(v) {}
    PropertyValue(const vec2& v) : type(Type::Float2), _float2(v) {}
    PropertyValue(const vec3& v) : type(Type::Float3), _float3(v) {}
    PropertyValue(const vec4& v) : type(Type::Float4), _float4(v) {}
    PropertyValue(const mat4& v) : type(Type::Matrix4), _matrix4(v) {}
    PropertyValue(const char* v) : type(Type::String), _string(v) {}
    PropertyValue(const std::string& v) : type(Type::String), _string(v) {}
    PropertyValue(const Strings& v) : type(Type::Strings) { _strings = v; }
    PropertyValue(std::nullptr_t) : type(Type::Undefined) {}

    Type type = Type::Undefined;

    const std::string& asString() const
    {
        AU_ASSERT(type == Type::String, "not a string");
        return _string;
    }
    bool asBool() const
    {
        AU_ASSERT(type == Type::Bool, "not a bool");
        return _bool;
    }
    int asInt() const
    {
        AU_ASSERT(type == Type::Int, "not an int");
        return _int;
    }
    float asFloat() const
    {
        AU_ASSERT(type == Type::Float, "not a float");
        return _float;
    }
    vec2 asFloat2() const
    {
        AU_ASSERT(type == Type::Float2, "not a float2");
        return _float2;
    }
    vec3 asFloat3() const
    {
        AU_ASSERT(type == Type::Float3, "not a float3");
        return _float3;
    }
    vec4 asFloat4() const
    {
        AU_ASSERT(type == Type::Float4, "not a float4");
        return _float4;
    }
    mat4 asMatrix4() const
    {
        AU_ASSERT(type == Type::Matrix4, "not a matrix4");
        return _matrix4;
    }
    Strings& asStrings()
    {
        AU_ASSERT(type == Type::Strings, "not a string array");
        return _strings;
    }
    const Strings& asStrings() const
    {
        AU_ASSERT(type == Type::Strings, "not a string array");
        return _strings;
    }
    bool hasValue() { return type != Type::Undefined; }
    void clear()
    {
        type = Type::Undefined;
        _string.clear();
        _strings.clear();
    }
    bool operator!=(const PropertyValue& in) const { return !(*this == in); }
    bool operator==(const PropertyValue& in) const
    {
        if (type != in.type)
            return false;
        switch (type)
        {
        case Type::Bool: return _bool == in._bool;
        case Type::Int: return _int == in._int;
        case Type::Float: return _float == in._float;
        case Type::Float2: return _float2 == in._float2;
        case Type::Float3: return _float3 == in._float3;
        case Type::Float4: return _float4 == in._float4;
        case Type::Matrix4: return _matrix4 == in._matrix4;
        case Type::String: return _string == in._string;
        case Type::Strings: return _strings == in._strings;
        default: return false;
        }
    }
    // Comma-separated components (a matrix column by column), the string, or the strings.
    std::string toString() const
    {
        auto join = [](const float* v, int n) {
            std::string s;
            for (int i = 0; i < n; i++)
                s += (i ? ", " : "") + std::to_string(v[i]);
            return s;
        };
        switch (type)
        {
        case Type::Bool: return std::to_string(_bool);
        case Type::Int: return std::to_string(_int);
        case Type::Float: return std::to_string(_float);
        case Type::Float2: return join(&_float2.x, 2);
        case Type::Float3: return join(&_float3.x, 3);
        case Type::Float4: return join(&_float4.x, 4);
        case Type::Matrix4: return join(&_matrix4[0].x, 16);
        case Type::String: return _string;
        case Type::Strings:
        {
            std::string s;
            for (size_t i = 0; i < _strings.size(); i++)
                s += (i ? ", " : "") + _strings[i];
            return s;
        }
        default: return "";
        }
    }

    union
    {
        bool _bool;
        int _int;
        float _float;
        vec2 _float2;
        vec3 _float3;
        vec4 _float4;
        mat4 _matrix4;
    };
    std::string _string;
    Strings _strings;
};

using Properties = std::map<std::string, PropertyValue>;

enum class AttributeFormat : uint8_t
{
    SInt8,
    UInt8,
    SInt16,
    UInt16,
    SInt32,
    UInt32,
    Float,
    Float2,
    Float3,
    Float4
};

// This backend renders Triangles (indexed or not).
enum class PrimitiveType : uint8_t
{
    Points,
    Lines,
    Linestrip,
    Triangles,
    Trianglestrip
};

// This backend takes Integer_RGBA, Float_RGBA and Float_RGB images and renders into Integer_RGBA
// and Float_RGBA targets.
enum class ImageFormat : uint8_t
{
    Byte_R,
    Integer_RGBA,
    Integer_RG,
    Integer_R,
    Short_RGBA,
    Half_RGBA,
    Float_RGBA,
    Float_RGB,
    Float_RG,
    Float_R
};

struct VertexDescription
{
    std::unordered_map<std::string, AttributeFormat> attributes;
    size_t count = 0;
    bool hasAttribute(const std::string& name) const { return attributes.count(name) != 0; }
};

struct AttributeData
{
    const void* address = nullptr;
    size_t offset       = 0;
    size_t size         = 0;
    size_t stride       = 0;
};

using AttributeDataMap = std::map<std::string, AttributeData>;

// Fills the attribute buffers (positions Float3, normals Float3, texture coordinates Float2, indices
// UInt32) when the renderer first needs the geometry; the renderer copies them.
using GetAttributeDataFunction = std::function<bool(AttributeDataMap& dataOut, size_t firstVertex,
    size_t vertexCount, size_t firstIndex, size_t indexCount)>;
// Called once the renderer has copied them.
using AttributeUpdateCompleteFunction = std::function<void(const AttributeDataMap& dataOut,
    size_t firstVertex, size_t vertexCount, size_t firstIndex, size_t indexCount)>;

struct GeometryDescriptor
{
    PrimitiveType type = PrimitiveType::Triangles;
    VertexDescription vertexDesc;
    size_t indexCount = 0;
    GetAttributeDataFunction getAttributeData               = nullptr;
    AttributeUpdateCompleteFunction attributeUpdateComplete = nullptr;
};

struct ImageData
{
    const void* pPixelBuffer = nullptr;
    size_t bytesPerRow       = 0;
    size_t bufferSize        = 0;
    glm::ivec2 dimensions    = glm::ivec2(0, 0);
    ImageFormat format       = ImageFormat::Integer_RGBA;
    bool overrideLinearize   = false;
    bool linearize           = true;
};

using AllocateBufferFunction = std::function<void*(size_t size)>;
using GetImageDataFunction   = std::function<bool(ImageData& dataOut, AllocateBufferFunction alloc)>;
using ImageUpdateCompleteFunction = std::function<void()>;

struct ImageDescriptor
{
    bool linearize     = true;
    bool isEnvironment = false;
    GetImageDataFunction getData               = nullptr;
    ImageUpdateCompleteFunction updateComplete = nullptr;
};

struct InstanceDefinition
{
    Path path;
    Properties properties;
};
using InstanceDefinitions = std::vector<InstanceDefinition>;
using Paths               = std::vector<Path>;

class AURORA_API IImage
{
public:
    struct InitData
    {
        const void* pImageData = nullptr;
        ImageFormat format     = ImageFormat::Integer_RGBA;
        bool linearize;
        bool isEnvironment = false;
        uint32_t width     = 0;
        uint32_t height    = 0;
        uint32_t depth     = 0;
        std::string name;
    };

protected:
    virtual ~IImage() = default;
};
MAKE_AURORA_PTR(IImage);

class AURORA_API ISampler
{
public:
    virtual ~ISampler() = default;
};
MAKE_AURORA_PTR(ISampler);

class AURORA_API IValues
{
public:
    enum class Type
    {
        Undefined,
        Boolean,
        Int,
        Float,
        Float2,
        Float3,
        Matrix,
        Image,
        Sampler,
        String
    };
    virtual void setBoolean(const std::string& name, bool value)               = 0;
    virtual void setInt(const std::string& name, int value)                    = 0;
    virtual void setFloat(const std::string& name, float value)                = 0;
    virtual void setFloat2(const std::string& name, const float* value)        = 0;
    virtual void setFloat3(const std::string& name, const float* value)        = 0;
    virtual void setMatrix(const std::string& name, const float* value)        = 0;
    virtual void setImage(const std::string& name, const IImagePtr& value)     = 0;
    virtual void setSampler(const std::string& name, const ISamplerPtr& value) = 0;
    virtual void setString(const std::string& name, const std::string& value)  = 0;
    virtual void clearValue(const std::string& name)                           = 0;
    virtual Type type(const std::string& name)                                 = 0;

protected:
    virtual ~IValues() = default;
};
MAKE_AURORA_PTR(IValues);

class AURORA_API ITarget
{
public:
    virtual void resize(uint32_t width, uint32_t height) = 0;

protected:
    virtual ~ITarget() = default;
};
MAKE_AURORA_PTR(ITarget);

using WindowHandle = void*;

// No window system here: createWindow returns null.
class AURORA_API IWindow : public ITarget
{
public:
    virtual void setVSyncEnabled(bool enabled) = 0;

protected:
    virtual ~IWindow() = default;
};
MAKE_AURORA_PTR(IWindow);

class AURORA_API IRenderBuffer : public ITarget
{
public:
    class IBuffer
    {
    public:
        virtual const void* data() = 0;
        virtual const void* handle() { return nullptr; }

    protected:
        IBuffer()          = default;
        virtual ~IBuffer() = default;
    };
    using IBufferPtr = std::shared_ptr<IRenderBuffer::IBuffer>;

    // Pixels of the last render (rows top to bottom); stride receives the bytes per row.
    virtual const void* data(size_t& stride, bool removePadding = false) = 0;
    // A copy of those pixels that later renders leave alone.
    virtual IBufferPtr asReadable(size_t& stride) = 0;
    // Shareable GPU memory: none here (null).
    virtual IBufferPtr asShared() = 0;

protected:
    virtual ~IRenderBuffer() = default;
};
MAKE_AURORA_PTR(IRenderBuffer);

class AURORA_API IGeometry
{
protected:
    virtual ~IGeometry() = default;
};
MAKE_AURORA_PTR(IGeometry);

// Environment values (Names::EnvironmentProperties); the scene takes environments by path
// (IScene::setEnvironmentProperties / setEnvironment).
class AURORA_API IEnvironment
{
public:
    virtual IValues& values() = 0;

protected:
    virtual ~IEnvironment() = default;
};
MAKE_AURORA_PTR(IEnvironment);

class AURORA_API IGroundPlane
{
public:
    virtual IValues& values() = 0;

protected:
    virtual ~IGroundPlane() = default;
};
MAKE_AURORA_PTR(IGroundPlane);

class AURORA_API IMaterial
{
public:
    virtual IValues& values() = 0;

protected:
    virtual ~IMaterial() = default;
};
MAKE_AURORA_PTR(IMaterial);

using LayerDefinition  = std::pair<IMaterialPtr, IGeometryPtr>;
using LayerDefinitions = std::vector<LayerDefinition>;

class AURORA_API IInstance
{
public:
    virtual void setMaterial(const IMaterialPtr& pMaterial) = 0;
    virtual void setTransform(const mat4& pTransform)       = 0;
    virtual void setObjectIdentifier(int objectId)          = 0;
    virtual void setVisible(bool visible)                   = 0;
    virtual IGeometryPtr geometry() const                   = 0;

protected:
    virtual ~IInstance() = default;
};
MAKE_AURORA_PTR(IInstance);

class AURORA_API ILight
{
public:
    virtual IValues& values() = 0;

protected:
    virtual ~ILight() = default;
};
MAKE_AURORA_PTR(ILight);

enum ResourceType
{
    Material = 0,
    Instance,
    Environment,
    Geometry,
    Sampler,
    GroundPlane,
    Image,
    Light,
    Invalid
};

class AURORA_API IScene
{
public:
    virtual ResourceType getResourceType(const Path& atPath) = 0;
    virtual void setImageDescriptor(const Path& atPath, const ImageDescriptor& desc) = 0;
    // PNG or Radiance HDR files, read when first used.
    virtual void setImageFromFilePath(const Path& atPath, const std::string& filePath = "",
        bool linearize = true, bool isEnvironment = false) = 0;
    virtual void setSamplerProperties(const Path& atPath, const Properties& props) = 0;
    virtual void setMaterialType(const Path& atPath,
        const std::string& materialType = Names::MaterialTypes::kBuiltIn,
        const std::string& document     = "Default") = 0;
    virtual void setGeometryDescriptor(const Path& atPath, const GeometryDescriptor& desc) = 0;
    // Resources stay resident here whether or not they are marked permanent.
    virtual void addPermanent(const Path& resource)    = 0;
    virtual void removePermanent(const Path& resource) = 0;
    virtual bool addInstance(const Path& atPath, const Path& geometry, const Properties& properties = {}) = 0;
    virtual Paths addInstances(const Path& geometry, const InstanceDefinitions& definitions) = 0;
    virtual bool setEnvironmentProperties(const Path& environment, const Properties& environmentProperties) = 0;
    virtual bool setEnvironment(const Path& environment) = 0;
    virtual void removeInstance(const Path& path)        = 0;
    virtual void removeInstances(const Paths& paths)     = 0;
    virtual void setMaterialProperties(const Path& path, const Properties& materialProperties) = 0;
    virtual void setInstanceProperties(const Path& path, const Properties& instanceProperties) = 0;
    virtual void setInstanceProperties(const Paths& paths, const Properties& instanceProperties) = 0;
    virtual void setBounds(const vec3& min, const vec3& max)     = 0;
    virtual void setBounds(const float* min, const float* max)   = 0;
    virtual void setGroundPlanePointer(const IGroundPlanePtr& pGroundPlane) = 0;
    virtual IInstancePtr addInstancePointer(const Path& path, const IGeometryPtr& geom,
        const IMaterialPtr& pMaterial, const mat4& pTransform, const LayerDefinitions& materialLayers = {}) = 0;
    virtual ILightPtr addLightPointer(const std::string& lightType) = 0;

protected:
    virtual ~IScene() = default;
};
MAKE_AURORA_PTR(IScene);

// This backend writes kFinal.
enum class AOV
{
    kFinal,
    kDepthNDC,
    kMotion,
    kDiffuseAlbedo,
    kSpecularAlbedo,
    kNormal,
    kRoughness
};
using TargetAssignments = std::unordered_map<AOV, ITargetPtr>;

class AURORA_API IRenderer
{
public:
    // Default selects this backend's CUDA path tracer; the reference's HGI and DirectX backends
    // are not part of this library (createRenderer returns null for them).
    enum class Backend
    {
        HGI,
        DirectX,
        Default
    };
    struct UpscalerSupport
    {
        bool isSupported              = false;
        bool needsDriverUpdate        = false;
        uint32_t minDriverVersionMajor = 0;
        uint32_t minDriverVersionMinor = 0;
    };

    virtual IWindowPtr createWindow(WindowHandle handle, uint32_t width, uint32_t height) = 0;
    virtual IRenderBufferPtr createRenderBuffer(int width, int height, ImageFormat format) = 0;
    virtual IImagePtr createImagePointer(const IImage::InitData& initData) = 0;
    virtual ISamplerPtr createSamplerPointer(const Properties& props) = 0;
    virtual IMaterialPtr createMaterialPointer(const std::string& materialType = Names::MaterialTypes::kBuiltIn,
        const std::string& document = "Default", const std::string& name = "") = 0;
    virtual IEnvironmentPtr createEnvironmentPointer() = 0;
    virtual IGeometryPtr createGeometryPointer(const GeometryDescriptor& desc, const std::string& name = "") = 0;
    virtual IGroundPlanePtr createGroundPlanePointer() = 0;
    virtual IScenePtr createScene() = 0;
    virtual void setOptions(const Properties& options) = 0;
    virtual IValues& options() = 0;
    virtual Backend backend() const = 0;
    virtual void setScene(const IScenePtr& pScene) = 0;
    virtual void setTargets(const TargetAssignments& targetAssignments) = 0;
    virtual void setCamera(const mat4& view, const mat4& projection, float focalDistance = 1.0f,
        float lensRadius = 0.0f) = 0;
    virtual void setCamera(const float* view, const float* proj, float focalDistance = 1.0f,
        float lensRadius = 0.0f) = 0;
    virtual void render(uint32_t sampleStart = 0, uint32_t sampleCount = 1) = 0;
    virtual void waitForTask() = 0;
    virtual const std::vector<std::string>& builtInMaterials() = 0;
    virtual void setLoadResourceFunction(LoadResourceFunction func) = 0;
    virtual void addMdlSearchPath(const std::string& path) = 0;
    // No upscaler here: only "None" is supported.
    virtual UpscalerSupport upscalerSupport(const std::string& mode)
    {
        return { mode == Names::UpscalerModes::kNone, false, 0, 0 };
    }

protected:
    virtual ~IRenderer() = default;
};
MAKE_AURORA_PTR(IRenderer);

// The renderer's logger is Aurora's Foundation library's (not part of this backend).
AURORA_API Foundation::Log& logger();

AURORA_API IRendererPtr createRenderer(
    IRenderer::Backend type = IRenderer::Backend::Default, uint32_t taskCount = 3);

} // namespace Aurora
