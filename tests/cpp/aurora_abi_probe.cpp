// Prints the binary interface of an Aurora public header (Aurora/Aurora.h): the vtable slot of
// every virtual function (read from its pointer to member, which the Itanium C++ ABI encodes as
// 1 + the slot's byte offset), the size and member offsets of every value type, and the values of
// every enumerator.  tests/test_aurora_dropin.py compiles it against the reference's own header
// and against this repository's, and requires identical output: a client compiled against either
// calls the same functions through the same slots on objects of the same layout.
#include <Aurora/Aurora.h>

#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstring>

using namespace Aurora;

template <class M>
long slot(M m)
{
    static_assert(sizeof(M) == 2 * sizeof(uintptr_t), "Itanium member pointer");
    uintptr_t raw[2];
    std::memcpy(raw, &m, sizeof raw);
    return (raw[0] & 1) ? long(raw[0] - 1) : -1;
}

#define V(cls, ret, name, ...) \
    std::printf("%s::%s(%s) slot %ld\n", #cls, #name, #__VA_ARGS__, slot(static_cast<ret (cls::*)(__VA_ARGS__)>(&cls::name)))
#define VC(cls, ret, name, ...) \
    std::printf("%s::%s(%s) const slot %ld\n", #cls, #name, #__VA_ARGS__, slot(static_cast<ret (cls::*)(__VA_ARGS__) const>(&cls::name)))
#define S(type) std::printf("sizeof %s %zu align %zu\n", #type, sizeof(type), alignof(type))
#define O(type, member) std::printf("offsetof %s.%s %zu\n", #type, #member, offsetof(type, member))
#define E(value) std::printf("%s = %d\n", #value, int(value))

int main()
{
    V(IValues, void, setBoolean, const std::string&, bool);
    V(IValues, void, setInt, const std::string&, int);
    V(IValues, void, setFloat, const std::string&, float);
    V(IValues, void, setFloat2, const std::string&, const float*);
    V(IValues, void, setFloat3, const std::string&, const float*);
    V(IValues, void, setMatrix, const std::string&, const float*);
    V(IValues, void, setImage, const std::string&, const IImagePtr&);
    V(IValues, void, setSampler, const std::string&, const ISamplerPtr&);
    V(IValues, void, setString, const std::string&, const std::string&);
    V(IValues, void, clearValue, const std::string&);
    V(IValues, IValues::Type, type, const std::string&);
    V(ITarget, void, resize, uint32_t, uint32_t);
    V(IWindow, void, setVSyncEnabled, bool);
    V(IRenderBuffer, const void*, data, size_t&, bool);
    V(IRenderBuffer, IRenderBuffer::IBufferPtr, asReadable, size_t&);
    V(IRenderBuffer, IRenderBuffer::IBufferPtr, asShared);
    V(IRenderBuffer::IBuffer, const void*, data);
    V(IRenderBuffer::IBuffer, const void*, handle);
    V(IEnvironment, IValues&, values);
    V(IGroundPlane, IValues&, values);
    V(IMaterial, IValues&, values);
    V(ILight, IValues&, values);
    V(IInstance, void, setMaterial, const IMaterialPtr&);
    V(IInstance, void, setTransform, const mat4&);
    V(IInstance, void, setObjectIdentifier, int);
    V(IInstance, void, setVisible, bool);
    VC(IInstance, IGeometryPtr, geometry);
    V(IScene, ResourceType, getResourceType, const Path&);
    V(IScene, void, setImageDescriptor, const Path&, const ImageDescriptor&);
    V(IScene, void, setImageFromFilePath, const Path&, const std::string&, bool, bool);
    V(IScene, void, setSamplerProperties, const Path&, const Properties&);
    V(IScene, void, setMaterialType, const Path&, const std::string&, const std::string&);
    V(IScene, void, setGeometryDescriptor, const Path&, const GeometryDescriptor&);
    V(IScene, void, addPermanent, const Path&);
    V(IScene, void, removePermanent, const Path&);
    V(IScene, bool, addInstance, const Path&, const Path&, const Properties&);
    V(IScene, Paths, addInstances, const Path&, const InstanceDefinitions&);
    V(IScene, bool, setEnvironmentProperties, const Path&, const Properties&);
    V(IScene, bool, setEnvironment, const Path&);
    V(IScene, void, removeInstance, const Path&);
    V(IScene, void, removeInstances, const Paths&);
    V(IScene, void, setMaterialProperties, const Path&, const Properties&);
    V(IScene, void, setInstanceProperties, const Path&, const Properties&);
    V(IScene, void, setInstanceProperties, const Paths&, const Properties&);
    V(IScene, void, setBounds, const vec3&, const vec3&);
    V(IScene, void, setBounds, const float*, const float*);
    V(IScene, void, setGroundPlanePointer, const IGroundPlanePtr&);
    V(IScene, IInstancePtr, addInstancePointer, const Path&, const IGeometryPtr&, const IMaterialPtr&, const mat4&,
        const LayerDefinitions&);
    V(IScene, ILightPtr, addLightPointer, const std::string&);
    V(IRenderer, IWindowPtr, createWindow, WindowHandle, uint32_t, uint32_t);
    V(IRenderer, IRenderBufferPtr, createRenderBuffer, int, int, ImageFormat);
    V(IRenderer, IImagePtr, createImagePointer, const IImage::InitData&);
    V(IRenderer, ISamplerPtr, createSamplerPointer, const Properties&);
    V(IRenderer, IMaterialPtr, createMaterialPointer, const std::string&, const std::string&, const std::string&);
    V(IRenderer, IEnvironmentPtr, createEnvironmentPointer);
    V(IRenderer, IGeometryPtr, createGeometryPointer, const GeometryDescriptor&, const std::string&);
    V(IRenderer, IGroundPlanePtr, createGroundPlanePointer);
    V(IRenderer, IScenePtr, createScene);
    V(IRenderer, void, setOptions, const Properties&);
    V(IRenderer, IValues&, options);
    VC(IRenderer, IRenderer::Backend, backend);
    V(IRenderer, void, setScene, const IScenePtr&);
    V(IRenderer, void, setTargets, const TargetAssignments&);
    V(IRenderer, void, setCamera, const mat4&, const mat4&, float, float);
    V(IRenderer, void, setCamera, const float*, const float*, float, float);
    V(IRenderer, void, render, uint32_t, uint32_t);
    V(IRenderer, void, waitForTask);
    V(IRenderer, const std::vector<std::string>&, builtInMaterials);
    V(IRenderer, void, setLoadResourceFunction, LoadResourceFunction);
    V(IRenderer, void, addMdlSearchPath, const std::string&);
    V(IRenderer, IRenderer::UpscalerSupport, upscalerSupport, const std::string&);

    S(PropertyValue);
    O(PropertyValue, type);
    O(PropertyValue, _matrix4);
    O(PropertyValue, _string);
    O(PropertyValue, _strings);
    S(vec2);
    S(vec3);
    S(vec4);
    S(mat4);
    S(VertexDescription);
    O(VertexDescription, attributes);
    O(VertexDescription, count);
    S(AttributeData);
    O(AttributeData, address);
    O(AttributeData, offset);
    O(AttributeData, size);
    O(AttributeData, stride);
    S(GeometryDescriptor);
    O(GeometryDescriptor, type);
    O(GeometryDescriptor, vertexDesc);
    O(GeometryDescriptor, indexCount);
    O(GeometryDescriptor, getAttributeData);
    O(GeometryDescriptor, attributeUpdateComplete);
    S(ImageData);
    O(ImageData, pPixelBuffer);
    O(ImageData, bytesPerRow);
    O(ImageData, bufferSize);
    O(ImageData, dimensions);
    O(ImageData, format);
    O(ImageData, overrideLinearize);
    O(ImageData, linearize);
    S(ImageDescriptor);
    O(ImageDescriptor, linearize);
    O(ImageDescriptor, isEnvironment);
    O(ImageDescriptor, getData);
    O(ImageDescriptor, updateComplete);
    S(InstanceDefinition);
    O(InstanceDefinition, path);
    O(InstanceDefinition, properties);
    S(IImage::InitData);
    O(IImage::InitData, pImageData);
    O(IImage::InitData, format);
    O(IImage::InitData, linearize);
    O(IImage::InitData, isEnvironment);
    O(IImage::InitData, width);
    O(IImage::InitData, height);
    O(IImage::InitData, depth);
    O(IImage::InitData, name);
    S(IRenderer::UpscalerSupport);
    O(IRenderer::UpscalerSupport, minDriverVersionMinor);

    E(PropertyValue::Type::Strings);
    E(PropertyValue::Type::Matrix4);
    E(AttributeFormat::UInt32);
    E(AttributeFormat::Float3);
    E(AttributeFormat::Float4);
    E(PrimitiveType::Triangles);
    E(ImageFormat::Integer_RGBA);
    E(ImageFormat::Float_RGBA);
    E(ImageFormat::Float_RGB);
    E(ImageFormat::Float_R);
    E(IValues::Type::String);
    E(IValues::Type::Image);
    E(ResourceType::Light);
    E(ResourceType::Invalid);
    E(AOV::kFinal);
    E(AOV::kRoughness);
    E(IRenderer::Backend::Default);
    return 0;
}
