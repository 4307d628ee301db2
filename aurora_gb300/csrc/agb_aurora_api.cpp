// Aurora's own public interface (include/Aurora/Aurora.h, declared as Libraries/Aurora/API/Aurora/
// Aurora.h) for the GB300 backend: Aurora::createRenderer and the IRenderer / IScene / IMaterial /
// IGeometry / IImage / ISampler / IEnvironment / IInstance / ILight / IGroundPlane /
// IRenderBuffer objects it hands out, implemented over the path-keyed C++ layer
// (aurora_gb300.hpp, agb_aurora.cpp), which itself renders through the C ABI.
//
// Path-keyed calls pass through with their values converted (Aurora's tagged PropertyValue to the
// layer's variant, glm matrices to column-major float arrays).  Objects made by the renderer's
// create*Pointer calls (materials, geometry, images, samplers) have no path of their own in
// Aurora; each gets one here ("/__aurora_pointer/<kind>/<n>") and is declared in a scene the first
// time an instance of that scene uses it (IScene::addInstancePointer).  A pointer material's later
// value changes reach the scenes it is declared in at the next render.
#include <Aurora/Aurora.h>

#include <atomic>
#include <cstring>
#include <set>

#include "aurora_gb300.hpp"

namespace Aurora
{
namespace Names
{
// The reference's values (Libraries/Aurora/Source/AuroraNames.cpp).
const std::string InstanceProperties::kGeometry("geometry");
const std::string InstanceProperties::kMaterial("material");
const std::string InstanceProperties::kTransform("transform");
const std::string InstanceProperties::kObjectID("objectID");
const std::string InstanceProperties::kVisible("visible");
const std::string InstanceProperties::kSelectable("selectable");
const std::string InstanceProperties::kMaterialLayers("layer_materials");
const std::string InstanceProperties::kGeometryLayers("layer_geometry");
const std::string EnvironmentProperties::kLightTop("light_top");
const std::string EnvironmentProperties::kLightBottom("light_bottom");
const std::string EnvironmentProperties::kLightImage("light_image");
const std::string EnvironmentProperties::kLightTransform("light_transform");
const std::string EnvironmentProperties::kBackgroundTop("background_top");
const std::string EnvironmentProperties::kBackgroundBottom("background_bottom");
const std::string EnvironmentProperties::kBackgroundImage("background_image");
const std::string EnvironmentProperties::kBackgroundTransform("background_transform");
const std::string EnvironmentProperties::kBackgroundUseScreen("background_use_screen");
const std::string AddressModes::kWrap("Wrap");
const std::string AddressModes::kMirror("Mirror");
const std::string AddressModes::kClamp("Clamp");
const std::string AddressModes::kBorder("Border");
const std::string AddressModes::kMirrorOnce("MirrorOnce");
const std::string SamplerProperties::kAddressModeU("AddressModeU");
const std::string SamplerProperties::kAddressModeV("AddressModeV");
const std::string VertexAttributes::kPosition("position");
const std::string VertexAttributes::kNormal("normal");
const std::string VertexAttributes::kTangent("tangent");
const std::string VertexAttributes::kTexCoord0("tcoord0");
const std::string VertexAttributes::kTexCoord1("tcoord1");
const std::string VertexAttributes::kTexCoord2("tcoord2");
const std::string VertexAttributes::kTexCoord3("tcoord3");
const std::string VertexAttributes::kTexCoord4("tcoord4");
const std::string VertexAttributes::kIndices("indices");
const std::string MaterialTypes::kBuiltIn("BuiltIn");
const std::string MaterialTypes::kMaterialX("MaterialX");
const std::string MaterialTypes::kMaterialXPath("MaterialXPath");
const std::string UpscalerModes::kNone("None");
const std::string UpscalerModes::kDLSS("DLSS");
const std::string UpscalerModes::kFSR("FSR");
const std::string UpscalerModes::kDLSSRayReconstruction("DLSSRayReconstruction");
const std::string LightTypes::kDistantLight("DistantLight");
const std::string LightProperties::kDirection("direction");
const std::string LightProperties::kAngularDiameter("angular_diameter_radians");
const std::string LightProperties::kExposure("exposure");
const std::string LightProperties::kIntensity("intensity");
const std::string LightProperties::kColor("color");
} // namespace Names
} // namespace Aurora

namespace agb_dropin
{
namespace A = Aurora;
namespace G = agb_aurora;

void report(const std::string& msg)
{
    std::fprintf(stderr, "aurora_gb300 (Aurora interface): %s\n", msg.c_str());
}

G::mat4 toInner(const A::mat4& m)
{
    G::mat4 r;
    std::memcpy(r.data(), &m[0].x, 16 * sizeof(float));
    return r;
}
G::mat4 toInner(const float* m)
{
    G::mat4 r;
    std::memcpy(r.data(), m, 16 * sizeof(float));
    return r;
}

// A property value in the C++ layer's kinds (an undefined value clears the property); false for
// a kind that layer has no use for (Float4).
bool toInner(const A::PropertyValue& v, G::PropertyValue& out)
{
    using T = A::PropertyValue::Type;
    switch (v.type)
    {
    case T::Undefined: out = std::monostate(); return true;
    case T::Bool: out = v._bool; return true;
    case T::Int: out = v._int; return true;
    case T::Float: out = v._float; return true;
    case T::Float2: out = G::vec2{ v._float2.x, v._float2.y }; return true;
    case T::Float3: out = G::vec3{ v._float3.x, v._float3.y, v._float3.z }; return true;
    case T::Matrix4: out = toInner(v._matrix4); return true;
    case T::String: out = v._string; return true;
    case T::Strings: out = v._strings; return true;
    default: return false;
    }
}

G::Properties toInner(const A::Properties& props, const std::string& where)
{
    G::Properties out;
    for (auto& kv : props)
    {
        G::PropertyValue v;
        if (toInner(kv.second, v))
            out[kv.first] = v;
        else
            report(where + ": property " + kv.first + " has a kind this backend does not take; ignored");
    }
    return out;
}

bool toInner(A::ImageFormat f, G::ImageFormat& out)
{
    switch (f)
    {
    case A::ImageFormat::Integer_RGBA: out = G::ImageFormat::Integer_RGBA; return true;
    case A::ImageFormat::Float_RGBA: out = G::ImageFormat::Float_RGBA; return true;
    case A::ImageFormat::Float_RGB: out = G::ImageFormat::Float_RGB; return true;
    default: return false;
    }
}

size_t bytesPerPixel(A::ImageFormat f)
{
    return f == A::ImageFormat::Integer_RGBA ? 4 : f == A::ImageFormat::Float_RGBA ? 16 : f == A::ImageFormat::Float_RGB ? 12 : 0;
}

// Aurora geometry descriptor -> the layer's (attribute buffers pass through field by field).
G::GeometryDescriptor toInner(const A::GeometryDescriptor& d, const std::string& where)
{
    G::GeometryDescriptor g;
    if (d.type != A::PrimitiveType::Triangles)
        report(where + ": only triangle geometry is rendered");
    for (auto& kv : d.vertexDesc.attributes)
    {
        if (kv.second == A::AttributeFormat::Float3)
            g.vertexDesc.attributes[kv.first] = G::AttributeFormat::Float3;
        else if (kv.second == A::AttributeFormat::Float2)
            g.vertexDesc.attributes[kv.first] = G::AttributeFormat::Float2;
        else if (kv.second == A::AttributeFormat::UInt32)
            g.vertexDesc.attributes[kv.first] = G::AttributeFormat::UInt;
        else
            report(where + ": attribute " + kv.first + " has a format this backend does not read; ignored");
    }
    g.vertexDesc.count = d.vertexDesc.count;
    g.indexCount       = d.indexCount;
    auto toOuter = [](const G::AttributeDataMap& in) {
        A::AttributeDataMap out;
        for (auto& kv : in)
            out[kv.first] = A::AttributeData{ kv.second.address, kv.second.offset, kv.second.size, kv.second.stride };
        return out;
    };
    if (d.getAttributeData)
    {
        A::GetAttributeDataFunction get = d.getAttributeData;
        g.getAttributeData = [get, toOuter](G::AttributeDataMap& buffers, size_t fv, size_t vc, size_t fi, size_t ic) {
            A::AttributeDataMap outer = toOuter(buffers);
            if (!get(outer, fv, vc, fi, ic))
                return false;
            for (auto& kv : outer)
            {
                G::AttributeData& a = buffers[kv.first];
                a.address           = kv.second.address;
                a.offset            = kv.second.offset;
                a.size              = kv.second.size;
                a.stride            = kv.second.stride;
            }
            return true;
        };
    }
    if (d.attributeUpdateComplete)
    {
        A::AttributeUpdateCompleteFunction done = d.attributeUpdateComplete;
        g.attributeUpdateComplete = [done, toOuter](const G::AttributeDataMap& buffers, size_t fv, size_t vc, size_t fi,
                                        size_t ic) { done(toOuter(buffers), fv, vc, fi, ic); };
    }
    return g;
}

// Aurora image descriptor -> the layer's: the client's buffer allocator is served from storage
// held until the renderer reports the upload complete.
G::ImageDescriptor toInner(const A::ImageDescriptor& d, const std::string& where)
{
    G::ImageDescriptor g;
    g.linearize = d.linearize;
    auto storage = std::make_shared<std::vector<uint8_t>>();
    A::GetImageDataFunction get = d.getData;
    A::ImageUpdateCompleteFunction done = d.updateComplete;
    if (get)
        g.getData = [get, storage, where](G::ImageData& out) {
            A::ImageData a;
            A::AllocateBufferFunction alloc = [storage](size_t n) -> void* {
                storage->resize(n);
                return storage->data();
            };
            if (!get(a, alloc))
                return false;
            G::ImageFormat f;
            if (!toInner(a.format, f))
            {
                report(where + ": image format not supported (Integer_RGBA, Float_RGBA and Float_RGB are)");
                return false;
            }
            out.pPixelBuffer  = a.pPixelBuffer;
            out.bytesPerRow   = a.bytesPerRow;
            out.bufferSize    = a.bufferSize;
            out.dimensions    = { a.dimensions.x, a.dimensions.y };
            out.format        = f;
            out.overrideLinearize = a.overrideLinearize;
            out.linearize     = a.linearize;
            return true;
        };
    g.updateComplete = [storage, done](const G::ImageData&) {
        std::vector<uint8_t>().swap(*storage);
        if (done)
            done();
    };
    return g;
}

// ----------------------------------------------------------------------------- values
// IValues over a value set of the C++ layer (lights, ground planes, renderer options).
class InnerValues : public A::IValues
{
public:
    explicit InnerValues(G::IValues* v) : inner(v) {}
    G::IValues* inner;
    std::map<std::string, Type> types;
    void setBoolean(const std::string& n, bool v) override { inner->setBoolean(n, v), types[n] = Type::Boolean; }
    void setInt(const std::string& n, int v) override { inner->setInt(n, v), types[n] = Type::Int; }
    void setFloat(const std::string& n, float v) override { inner->setFloat(n, v), types[n] = Type::Float; }
    void setFloat2(const std::string& n, const float*) override { report("value " + n + ": float2 values are not taken here"); }
    void setFloat3(const std::string& n, const float* v) override
    {
        inner->setFloat3(n, G::vec3{ v[0], v[1], v[2] });
        types[n] = Type::Float3;
    }
    void setMatrix(const std::string& n, const float* v) override
    {
        inner->setMatrix(n, toInner(v));
        types[n] = Type::Matrix;
    }
    void setImage(const std::string& n, const A::IImagePtr&) override { report("value " + n + ": images are not taken here"); }
    void setSampler(const std::string& n, const A::ISamplerPtr&) override
    {
        report("value " + n + ": samplers are not taken here");
    }
    void setString(const std::string& n, const std::string& v) override { inner->setString(n, v), types[n] = Type::String; }
    void clearValue(const std::string& n) override
    {
        inner->clearValue(n);
        types.erase(n);
    }
    Type type(const std::string& n) override
    {
        auto it = types.find(n);
        return it == types.end() ? Type::Undefined : it->second;
    }
};

class Image;
class Sampler;

// IValues kept here (pointer materials, environments): properties, image and sampler objects.
class StoredValues : public A::IValues
{
public:
    A::Properties props;
    std::map<std::string, std::shared_ptr<Image>> images;
    std::map<std::string, std::shared_ptr<Sampler>> samplers;
    std::map<std::string, Type> types;
    std::set<std::string> cleared; // sent as undefined values, so the defaults apply again
    uint64_t version = 1;
    void set(const std::string& n, const A::PropertyValue& v, Type t)
    {
        props[n] = v;
        types[n] = t;
        cleared.erase(n);
        version++;
    }
    void setBoolean(const std::string& n, bool v) override { set(n, v, Type::Boolean); }
    void setInt(const std::string& n, int v) override { set(n, v, Type::Int); }
    void setFloat(const std::string& n, float v) override { set(n, v, Type::Float); }
    void setFloat2(const std::string& n, const float* v) override { set(n, A::vec2(v[0], v[1]), Type::Float2); }
    void setFloat3(const std::string& n, const float* v) override { set(n, A::vec3(v[0], v[1], v[2]), Type::Float3); }
    void setMatrix(const std::string& n, const float* v) override
    {
        A::mat4 m;
        std::memcpy(&m[0].x, v, 16 * sizeof(float));
        set(n, m, Type::Matrix);
    }
    void setImage(const std::string& n, const A::IImagePtr& v) override;
    void setSampler(const std::string& n, const A::ISamplerPtr& v) override;
    void setString(const std::string& n, const std::string& v) override { set(n, v, Type::String); }
    void clearValue(const std::string& n) override
    {
        props.erase(n);
        images.erase(n);
        samplers.erase(n);
        types.erase(n);
        cleared.insert(n);
        version++;
    }
    Type type(const std::string& n) override
    {
        auto it = types.find(n);
        return it == types.end() ? Type::Undefined : it->second;
    }
};

std::atomic<uint64_t> g_pointerId{ 1 };
std::string pointerPath(const char* kind)
{
    return std::string("/__aurora_pointer/") + kind + "/" + std::to_string(g_pointerId++);
}

// ------------------------------------------------------------------- pointer objects
class Image : public A::IImage
{
public:
    std::string path = pointerPath("image");
    A::ImageFormat format;
    bool linearize;
    uint32_t width, height;
    std::vector<uint8_t> pixels;
    A::ImageDescriptor descriptor() const
    {
        A::ImageDescriptor d;
        d.linearize     = linearize;
        auto self       = this;
        d.getData       = [self](A::ImageData& out, A::AllocateBufferFunction) {
            out.pPixelBuffer = self->pixels.data();
            out.bytesPerRow  = size_t(self->width) * bytesPerPixel(self->format);
            out.bufferSize   = self->pixels.size();
            out.dimensions   = glm::ivec2(int(self->width), int(self->height));
            out.format       = self->format;
            return true;
        };
        return d;
    }
};

class Sampler : public A::ISampler
{
public:
    std::string path = pointerPath("sampler");
    A::Properties props;
};

void StoredValues::setImage(const std::string& n, const A::IImagePtr& v)
{
    auto im = std::dynamic_pointer_cast<Image>(v);
    if (v && !im)
    {
        report("value " + n + ": not an image of this renderer");
        return;
    }
    if (im)
    {
        images[n] = im;
        types[n]  = Type::Image;
        cleared.erase(n);
    }
    else
    {
        images.erase(n);
        types.erase(n);
        cleared.insert(n);
    }
    version++;
}

void StoredValues::setSampler(const std::string& n, const A::ISamplerPtr& v)
{
    auto s = std::dynamic_pointer_cast<Sampler>(v);
    if (v && !s)
    {
        report("value " + n + ": not a sampler of this renderer");
        return;
    }
    if (s)
    {
        samplers[n] = s;
        types[n]    = Type::Sampler;
        cleared.erase(n);
    }
    else
    {
        samplers.erase(n);
        types.erase(n);
        cleared.insert(n);
    }
    version++;
}

class Material : public A::IMaterial
{
public:
    std::string path = pointerPath("material");
    std::string type, document;
    StoredValues vals;
    A::IValues& values() override { return vals; }
};

class Geometry : public A::IGeometry
{
public:
    std::string path = pointerPath("geometry");
    A::GeometryDescriptor desc;
};

class Environment : public A::IEnvironment
{
public:
    StoredValues vals;
    A::IValues& values() override { return vals; }
};

class Light : public A::ILight
{
public:
    explicit Light(G::ILightPtr l) : inner(std::move(l)), vals(&inner->values()) {}
    G::ILightPtr inner;
    InnerValues vals;
    A::IValues& values() override { return vals; }
};

class GroundPlane : public A::IGroundPlane
{
public:
    explicit GroundPlane(G::IGroundPlanePtr g) : inner(std::move(g)), vals(&inner->values()) {}
    G::IGroundPlanePtr inner;
    InnerValues vals;
    A::IValues& values() override { return vals; }
};

class Buffer : public A::IRenderBuffer::IBuffer
{
public:
    explicit Buffer(G::IRenderBuffer::IBufferPtr b) : inner(std::move(b)) {}
    G::IRenderBuffer::IBufferPtr inner;
    const void* data() override { return inner->data(); }
    const void* handle() override { return inner->handle(); }
};

class RenderBuffer : public A::IRenderBuffer
{
public:
    RenderBuffer(std::weak_ptr<G::IRenderer> r, G::IRenderBufferPtr b, G::ImageFormat f)
        : renderer(std::move(r)), inner(std::move(b)), format(f)
    {
    }
    std::weak_ptr<G::IRenderer> renderer;
    G::IRenderBufferPtr inner;
    G::ImageFormat format;
    void resize(uint32_t w, uint32_t h) override
    {
        if (auto r = renderer.lock())
            inner = r->createRenderBuffer(int(w), int(h), format);
    }
    const void* data(size_t& stride, bool removePadding) override { return inner->data(stride, removePadding); }
    IBufferPtr asReadable(size_t& stride) override
    {
        auto b = inner->asReadable(stride);
        return b ? std::make_shared<Buffer>(b) : nullptr;
    }
    IBufferPtr asShared() override
    {
        auto b = inner->asShared();
        return b ? std::make_shared<Buffer>(b) : nullptr;
    }
};

class Scene;

class Instance : public A::IInstance
{
public:
    std::weak_ptr<Scene> scene;
    std::string path;
    A::IGeometryPtr geom;
    void setMaterial(const A::IMaterialPtr& m) override;
    void setTransform(const A::mat4& t) override;
    void setObjectIdentifier(int id) override;
    void setVisible(bool visible) override;
    A::IGeometryPtr geometry() const override { return geom; }
};

// --------------------------------------------------------------------------------- scene
class Scene : public A::IScene, public std::enable_shared_from_this<Scene>
{
public:
    explicit Scene(G::IScenePtr s) : inner(std::move(s)) {}
    G::IScenePtr inner;
    std::map<std::string, A::ResourceType> kinds;
    std::set<std::string> declared;                                    // pointer objects declared here
    std::map<std::string, std::pair<std::weak_ptr<Material>, uint64_t>> materials; // and their versions

    A::ResourceType getResourceType(const A::Path& p) override
    {
        auto it = kinds.find(p);
        return it == kinds.end() ? A::ResourceType::Invalid : it->second;
    }
    void setImageDescriptor(const A::Path& p, const A::ImageDescriptor& d) override
    {
        inner->setImageDescriptor(p, toInner(d, "image " + p));
        kinds[p] = A::ResourceType::Image;
    }
    void setImageFromFilePath(const A::Path& p, const std::string& file, bool linearize, bool isEnvironment) override
    {
        inner->setImageFromFilePath(p, file, linearize, isEnvironment);
        kinds[p] = A::ResourceType::Image;
    }
    void setSamplerProperties(const A::Path& p, const A::Properties& props) override
    {
        inner->setSamplerProperties(p, toInner(props, "sampler " + p));
        kinds[p] = A::ResourceType::Sampler;
    }
    void setMaterialType(const A::Path& p, const std::string& type, const std::string& document) override
    {
        inner->setMaterialType(p, type, document);
        kinds[p] = A::ResourceType::Material;
    }
    void setGeometryDescriptor(const A::Path& p, const A::GeometryDescriptor& d) override
    {
        inner->setGeometryDescriptor(p, toInner(d, "geometry " + p));
        kinds[p] = A::ResourceType::Geometry;
    }
    void addPermanent(const A::Path&) override {}
    void removePermanent(const A::Path&) override {}
    bool addInstance(const A::Path& p, const A::Path& geometry, const A::Properties& props) override
    {
        bool ok = inner->addInstance(p, geometry, toInner(props, "instance " + p));
        if (ok)
            kinds[p] = A::ResourceType::Instance;
        return ok;
    }
    A::Paths addInstances(const A::Path& geometry, const A::InstanceDefinitions& defs) override
    {
        A::Paths out;
        for (const A::InstanceDefinition& d : defs)
            if (addInstance(d.path, geometry, d.properties))
                out.push_back(d.path);
        return out;
    }
    bool setEnvironmentProperties(const A::Path& p, const A::Properties& props) override
    {
        kinds[p] = A::ResourceType::Environment;
        return inner->setEnvironmentProperties(p, toInner(props, "environment " + p));
    }
    bool setEnvironment(const A::Path& p) override { return inner->setEnvironment(p); }
    void removeInstance(const A::Path& p) override
    {
        inner->removeInstance(p);
        kinds.erase(p);
    }
    void removeInstances(const A::Paths& paths) override
    {
        for (const A::Path& p : paths)
            removeInstance(p);
    }
    void setMaterialProperties(const A::Path& p, const A::Properties& props) override
    {
        inner->setMaterialProperties(p, toInner(props, "material " + p));
        kinds[p] = A::ResourceType::Material;
    }
    void setInstanceProperties(const A::Path& p, const A::Properties& props) override
    {
        inner->setInstanceProperties(p, toInner(props, "instance " + p));
    }
    void setInstanceProperties(const A::Paths& paths, const A::Properties& props) override
    {
        G::Properties g = toInner(props, "instances");
        for (const A::Path& p : paths)
            inner->setInstanceProperties(p, g);
    }
    void setBounds(const A::vec3& mn, const A::vec3& mx) override
    {
        inner->setBounds(G::vec3{ mn.x, mn.y, mn.z }, G::vec3{ mx.x, mx.y, mx.z });
    }
    void setBounds(const float* mn, const float* mx) override
    {
        inner->setBounds(G::vec3{ mn[0], mn[1], mn[2] }, G::vec3{ mx[0], mx[1], mx[2] });
    }
    void setGroundPlanePointer(const A::IGroundPlanePtr& g) override
    {
        auto gp = std::dynamic_pointer_cast<GroundPlane>(g);
        if (g && !gp)
            throw G::Error("setGroundPlanePointer: not a ground plane of this renderer");
        inner->setGroundPlanePointer(gp ? gp->inner : nullptr);
        kinds["/__aurora_ground_plane"] = A::ResourceType::GroundPlane;
    }
    // Declares a pointer geometry, material (with its images and samplers) in this scene.
    std::string declare(const A::IGeometryPtr& g)
    {
        auto geom = std::dynamic_pointer_cast<Geometry>(g);
        if (!geom)
            throw G::Error("addInstancePointer: not a geometry of this renderer");
        if (declared.insert(geom->path).second)
            setGeometryDescriptor(geom->path, geom->desc);
        return geom->path;
    }
    std::string declare(const A::IMaterialPtr& m)
    {
        auto mat = std::dynamic_pointer_cast<Material>(m);
        if (!mat)
            throw G::Error("addInstancePointer: not a material of this renderer");
        if (declared.insert(mat->path).second)
            setMaterialType(mat->path, mat->type, mat->document);
        apply(mat);
        return mat->path;
    }
    // (Re-)applies a pointer material's values when they changed since it was last applied.
    void apply(const std::shared_ptr<Material>& mat)
    {
        auto& slot = materials[mat->path];
        if (slot.second == mat->vals.version)
            return;
        A::Properties props = mat->vals.props;
        for (const std::string& n : mat->vals.cleared)
            props[n] = nullptr;
        for (auto& kv : mat->vals.images)
        {
            if (declared.insert(kv.second->path).second)
                setImageDescriptor(kv.second->path, kv.second->descriptor());
            props[kv.first] = kv.second->path;
        }
        for (auto& kv : mat->vals.samplers)
        {
            if (declared.insert(kv.second->path).second)
                setSamplerProperties(kv.second->path, kv.second->props);
            props[kv.first] = kv.second->path;
        }
        setMaterialProperties(mat->path, props);
        slot = { mat, mat->vals.version };
    }
    void syncMaterials()
    {
        for (auto it = materials.begin(); it != materials.end();)
        {
            auto m = it->second.first.lock();
            if (!m)
            {
                it = materials.erase(it);
                continue;
            }
            ++it;
            apply(m);
        }
    }
    A::IInstancePtr addInstancePointer(const A::Path& p, const A::IGeometryPtr& geom, const A::IMaterialPtr& material,
        const A::mat4& transform, const A::LayerDefinitions& layers) override
    {
        A::Properties props;
        props[A::Names::InstanceProperties::kTransform] = transform;
        if (material)
            props[A::Names::InstanceProperties::kMaterial] = declare(material);
        if (!layers.empty())
        {
            A::Strings lm, lg;
            for (const A::LayerDefinition& l : layers)
            {
                lm.push_back(declare(l.first));
                lg.push_back(declare(l.second));
            }
            props[A::Names::InstanceProperties::kMaterialLayers] = lm;
            props[A::Names::InstanceProperties::kGeometryLayers] = lg;
        }
        if (!addInstance(p, declare(geom), props))
            return nullptr;
        auto inst   = std::make_shared<Instance>();
        inst->scene = shared_from_this();
        inst->path  = p;
        inst->geom  = geom;
        return inst;
    }
    A::ILightPtr addLightPointer(const std::string& type) override
    {
        auto l = inner->addLightPointer(type);
        kinds["/__aurora_light/" + std::to_string(g_pointerId++)] = A::ResourceType::Light;
        return l ? std::make_shared<Light>(l) : nullptr;
    }
};

void Instance::setMaterial(const A::IMaterialPtr& m)
{
    if (auto sc = scene.lock())
    {
        A::Properties props;
        props[A::Names::InstanceProperties::kMaterial] = m ? sc->declare(m) : std::string();
        sc->setInstanceProperties(path, props);
    }
}
void Instance::setTransform(const A::mat4& t)
{
    if (auto sc = scene.lock())
        sc->setInstanceProperties(path, A::Properties{ { A::Names::InstanceProperties::kTransform, t } });
}
void Instance::setObjectIdentifier(int id)
{
    if (auto sc = scene.lock())
        sc->setInstanceProperties(path, A::Properties{ { A::Names::InstanceProperties::kObjectID, id } });
}
void Instance::setVisible(bool visible)
{
    if (auto sc = scene.lock())
        sc->setInstanceProperties(path, A::Properties{ { A::Names::InstanceProperties::kVisible, visible } });
}

// ------------------------------------------------------------------------------ renderer
class Renderer : public A::IRenderer
{
public:
    explicit Renderer(G::IRendererPtr r) : inner(std::move(r)), optionValues(&inner->options()) {}
    G::IRendererPtr inner;
    InnerValues optionValues;
    std::shared_ptr<Scene> scene;
    A::TargetAssignments targets;

    A::IWindowPtr createWindow(A::WindowHandle, uint32_t, uint32_t) override { return nullptr; }
    A::IRenderBufferPtr createRenderBuffer(int w, int h, A::ImageFormat f) override
    {
        G::ImageFormat g;
        if (!toInner(f, g) || f == A::ImageFormat::Float_RGB)
        {
            report("createRenderBuffer: targets are Integer_RGBA or Float_RGBA");
            return nullptr;
        }
        auto b = inner->createRenderBuffer(w, h, g);
        return b ? std::make_shared<RenderBuffer>(inner, b, g) : nullptr;
    }
    A::IImagePtr createImagePointer(const A::IImage::InitData& d) override
    {
        size_t bpp = bytesPerPixel(d.format);
        if (!bpp || !d.pImageData || d.width == 0 || d.height == 0)
        {
            report("createImagePointer: Integer_RGBA, Float_RGBA or Float_RGB pixels required");
            return nullptr;
        }
        auto im       = std::make_shared<Image>();
        im->format    = d.format;
        im->linearize = d.linearize;
        im->width     = d.width;
        im->height    = d.height;
        const uint8_t* src = static_cast<const uint8_t*>(d.pImageData);
        im->pixels.assign(src, src + size_t(d.width) * d.height * bpp);
        return im;
    }
    A::ISamplerPtr createSamplerPointer(const A::Properties& props) override
    {
        auto s   = std::make_shared<Sampler>();
        s->props = props;
        return s;
    }
    A::IMaterialPtr createMaterialPointer(const std::string& type, const std::string& document, const std::string&) override
    {
        auto m      = std::make_shared<Material>();
        m->type     = type;
        m->document = document;
        return m;
    }
    A::IEnvironmentPtr createEnvironmentPointer() override { return std::make_shared<Environment>(); }
    A::IGeometryPtr createGeometryPointer(const A::GeometryDescriptor& desc, const std::string&) override
    {
        auto g  = std::make_shared<Geometry>();
        g->desc = desc;
        return g;
    }
    A::IGroundPlanePtr createGroundPlanePointer() override
    {
        auto g = inner->createGroundPlanePointer();
        return g ? std::make_shared<GroundPlane>(g) : nullptr;
    }
    A::IScenePtr createScene() override
    {
        auto s = inner->createScene();
        return s ? std::make_shared<Scene>(s) : nullptr;
    }
    void setOptions(const A::Properties& options) override { inner->setOptions(toInner(options, "options")); }
    A::IValues& options() override { return optionValues; }
    Backend backend() const override { return Backend::Default; }
    void setScene(const A::IScenePtr& s) override
    {
        auto sc = std::dynamic_pointer_cast<Scene>(s);
        if (s && !sc)
            throw G::Error("setScene: not a scene of this renderer");
        scene = sc;
        inner->setScene(sc ? sc->inner : nullptr);
    }
    void setTargets(const A::TargetAssignments& t) override
    {
        targets = t;
        applyTargets();
    }
    void applyTargets()
    {
        G::TargetAssignments g;
        for (auto& kv : targets)
        {
            if (kv.first != A::AOV::kFinal)
            {
                report("setTargets: only the final image (AOV::kFinal) is written");
                continue;
            }
            auto rb = std::dynamic_pointer_cast<RenderBuffer>(kv.second);
            if (kv.second && !rb)
                throw G::Error("setTargets: not a render buffer of this renderer");
            if (rb)
                g[G::AOV::Final] = rb->inner;
        }
        inner->setTargets(g);
    }
    void setCamera(const A::mat4& view, const A::mat4& proj, float focalDistance, float lensRadius) override
    {
        inner->setCamera(toInner(view), toInner(proj), focalDistance, lensRadius);
    }
    void setCamera(const float* view, const float* proj, float focalDistance, float lensRadius) override
    {
        inner->setCamera(toInner(view), toInner(proj), focalDistance, lensRadius);
    }
    void render(uint32_t sampleStart, uint32_t sampleCount) override
    {
        if (scene)
            scene->syncMaterials();
        applyTargets(); // a resized target holds a new buffer
        inner->render(sampleStart, sampleCount);
    }
    void waitForTask() override { inner->waitForTask(); }
    const std::vector<std::string>& builtInMaterials() override { return inner->builtInMaterials(); }
    void setLoadResourceFunction(A::LoadResourceFunction f) override { inner->setLoadResourceFunction(std::move(f)); }
    void addMdlSearchPath(const std::string&) override {}
};

} // namespace agb_dropin

namespace Aurora
{

IRendererPtr createRenderer(IRenderer::Backend type, uint32_t taskCount)
{
    if (type != IRenderer::Backend::Default)
        return nullptr; // the HGI and DirectX backends are not part of this library
    auto inner = agb_aurora::createRenderer(agb_aurora::IRenderer::Backend::CUDA, taskCount);
    return inner ? std::make_shared<agb_dropin::Renderer>(inner) : nullptr;
}

} // namespace Aurora
