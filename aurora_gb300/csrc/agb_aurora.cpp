// Implementation of the Aurora-style C++ interface (include/aurora_gb300.hpp) over the C ABI.
//
// The scene keeps Aurora's path-keyed, lazily activated resources (SceneBase.cpp): descriptors and
// properties are recorded when set, and the first render that needs them pulls geometry and image
// data through the client's callbacks, uploads them, and calls the completion callbacks so the
// client may free its buffers (GeometryBase.cpp:94-112).  Frame data follows
// RendererBase::updateFrameDataGPUStruct (RendererBase.cpp:225-295) and the HGI backend's choices
// (opaque shadows, HGIRenderer.cpp:491); post-processing follows RendererBase.cpp:297-337.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <list>
#include <mutex>
#include <set>

#include "agb.h"
#include "aurora_gb300.hpp"
#include "aurora_gb300_loaders.hpp"

namespace agb_aurora
{
namespace
{

std::mutex g_logMutex;
std::function<void(const std::string&)> g_log;

void logError(const std::string& msg)
{
    std::lock_guard<std::mutex> g(g_logMutex);
    if (g_log)
        g_log(msg);
    else
        std::fprintf(stderr, "aurora_gb300: %s\n", msg.c_str());
}

void check(agb_status st, const std::string& what)
{
    if (st != AGB_OK)
        throw Error(what + ": " + agb_last_error());
}

// Sets `src`'s values in `dst`; an undefined value (std::monostate) removes the property, so its
// default applies again.
void merge(Properties& dst, const Properties& src)
{
    for (auto& kv : src)
    {
        if (std::holds_alternative<std::monostate>(kv.second))
            dst.erase(kv.first);
        else
            dst[kv.first] = kv.second;
    }
}

template <class T>
const T* find(const Properties& p, const std::string& name)
{
    auto it = p.find(name);
    return it == p.end() ? nullptr : std::get_if<T>(&it->second);
}

// glm column-major mat4 -> the 3x4 rows of the matrix (object_to_world).
void rows3x4(const mat4& m, float out[12])
{
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 4; c++)
            out[4 * r + c] = m[4 * c + r];
}

// Row-major copy (the bytes of glm transpose(m)).
void rowMajor(const mat4& m, float out[16])
{
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++)
            out[4 * r + c] = m[4 * c + r];
}

// Inverse of a column-major 4x4 (double precision, rounded to float), column-major out.
bool inverse4(const mat4& m, mat4& out)
{
    double a[4][8];
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++)
        {
            a[r][c]     = m[4 * c + r];
            a[r][c + 4] = r == c ? 1.0 : 0.0;
        }
    for (int c = 0; c < 4; c++)
    {
        int p = c;
        for (int r = c + 1; r < 4; r++)
            if (std::fabs(a[r][c]) > std::fabs(a[p][c]))
                p = r;
        if (std::fabs(a[p][c]) < 1e-300)
            return false;
        if (p != c)
            for (int k = 0; k < 8; k++)
                std::swap(a[p][k], a[c][k]);
        double inv = 1.0 / a[c][c];
        for (int k = 0; k < 8; k++)
            a[c][k] *= inv;
        for (int r = 0; r < 4; r++)
            if (r != c)
            {
                double f = a[r][c];
                for (int k = 0; k < 8; k++)
                    a[r][k] -= f * a[c][k];
            }
    }
    for (int r = 0; r < 4; r++)
        for (int c = 0; c < 4; c++)
            out[4 * c + r] = float(a[r][c + 4]);
    return true;
}

const mat4 kIdentity = { 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1 };

class Values : public IValues
{
public:
    Properties props;
    bool dirty = true;
    void setBoolean(const std::string& n, bool v) override { props[n] = v; dirty = true; }
    void setInt(const std::string& n, int v) override { props[n] = v; dirty = true; }
    void setFloat(const std::string& n, float v) override { props[n] = v; dirty = true; }
    void setFloat3(const std::string& n, const vec3& v) override { props[n] = v; dirty = true; }
    void setMatrix(const std::string& n, const mat4& v) override { props[n] = v; dirty = true; }
    void setString(const std::string& n, const std::string& v) override { props[n] = v; dirty = true; }
    void clearValue(const std::string& n) override { props.erase(n); dirty = true; }
    float asFloat(const std::string& n, float def) const
    {
        if (auto* f = find<float>(props, n))
            return *f;
        if (auto* i = find<int>(props, n))
            return float(*i);
        return def;
    }
    int asInt(const std::string& n, int def) const
    {
        if (auto* i = find<int>(props, n))
            return *i;
        if (auto* f = find<float>(props, n))
            return int(*f);
        return def;
    }
    bool asBool(const std::string& n, bool def) const
    {
        if (auto* b = find<bool>(props, n))
            return *b;
        if (auto* i = find<int>(props, n))
            return *i != 0;
        return def;
    }
    vec3 asFloat3(const std::string& n, const vec3& def) const
    {
        auto* v = find<vec3>(props, n);
        return v ? *v : def;
    }
};

class Light : public ILight
{
public:
    Values v;
    Light()
    {
        // Distant-light defaults (HGI/HGILight.cpp:31-38): direction normalize(-1, -0.5, -1).
        float l = std::sqrt(1.f + 0.25f + 1.f);
        v.setFloat3(Names::LightProperties::kDirection, { -1.f / l, -0.5f / l, -1.f / l });
        v.setFloat3(Names::LightProperties::kColor, { 1.f, 1.f, 1.f });
        v.setFloat(Names::LightProperties::kAngularDiameter, 0.1f);
        v.setFloat(Names::LightProperties::kIntensity, 1.f);
    }
    IValues& values() override { return v; }
};

class GroundPlane : public IGroundPlane
{
public:
    Values v;
    GroundPlane()
    {
        // PTGroundPlane.cpp:42-51.
        v.setBoolean("enabled", true);
        v.setFloat3("position", { 0.f, 0.f, 0.f });
        v.setFloat3("normal", { 0.f, 1.f, 0.f });
        v.setFloat("shadow_opacity", 1.f);
        v.setFloat3("shadow_color", { 0.f, 0.f, 0.f });
        v.setFloat("reflection_opacity", 0.5f);
        v.setFloat3("reflection_color", { 0.5f, 0.5f, 0.5f });
        v.setFloat("reflection_roughness", 0.1f);
    }
    IValues& values() override { return v; }
    agb_ground_plane data() const
    {
        agb_ground_plane g{};
        g.enabled = v.asBool("enabled", true) ? 1 : 0;
        vec3 p = v.asFloat3("position", { 0.f, 0.f, 0.f }), n = v.asFloat3("normal", { 0.f, 1.f, 0.f });
        vec3 sc = v.asFloat3("shadow_color", { 0.f, 0.f, 0.f });
        vec3 rc = v.asFloat3("reflection_color", { 0.5f, 0.5f, 0.5f });
        for (int k = 0; k < 3; k++)
        {
            g.position[k]         = p[k];
            g.normal[k]           = n[k];
            g.shadow_color[k]     = sc[k];
            g.reflection_color[k] = rc[k];
        }
        g.shadow_opacity       = v.asFloat("shadow_opacity", 1.f);
        g.reflection_opacity   = v.asFloat("reflection_opacity", 0.5f);
        g.reflection_roughness = v.asFloat("reflection_roughness", 0.1f);
        return g;
    }
};

class RenderBuffer : public IRenderBuffer
{
public:
    int w, h;
    ImageFormat format;
    std::vector<uint8_t> rgba8;
    std::vector<float> rgba32;
    RenderBuffer(int width, int height, ImageFormat f) : w(width), h(height), format(f)
    {
        if (f == ImageFormat::Integer_RGBA)
            rgba8.assign(size_t(w) * h * 4, 0);
        else
            rgba32.assign(size_t(w) * h * 4, 0.f);
    }
    IBufferPtr asReadable(size_t& stride) override
    {
        struct Copy : IBuffer
        {
            std::vector<uint8_t> bytes;
            const void* data() override { return bytes.data(); }
        };
        auto c           = std::make_shared<Copy>();
        const void* src  = data(stride, false);
        size_t n         = stride * size_t(h);
        c->bytes.assign(static_cast<const uint8_t*>(src), static_cast<const uint8_t*>(src) + n);
        return c;
    }
    IBufferPtr asShared() override { return nullptr; }
    const void* data(size_t& stride, bool) override
    {
        stride = size_t(w) * (format == ImageFormat::Integer_RGBA ? 4 : 16);
        return format == ImageFormat::Integer_RGBA ? static_cast<const void*>(rgba8.data())
                                                   : static_cast<const void*>(rgba32.data());
    }
    int width() const override { return w; }
    int height() const override { return h; }
};

// Standard Surface property name -> (offset in agb_material in floats, component count).
struct MatField
{
    const char* name;
    size_t offset;
    int count;
    bool integer;
};
#define AGB_MF(field, n, i) { #field, offsetof(agb_material, field), n, i }
const MatField kMatFields[] = {
    AGB_MF(base, 1, false), AGB_MF(base_color, 3, false), AGB_MF(diffuse_roughness, 1, false),
    AGB_MF(metalness, 1, false), AGB_MF(specular, 1, false), AGB_MF(specular_color, 3, false),
    AGB_MF(specular_roughness, 1, false), AGB_MF(specular_IOR, 1, false),
    AGB_MF(specular_anisotropy, 1, false), AGB_MF(specular_rotation, 1, false),
    AGB_MF(transmission, 1, false), AGB_MF(transmission_color, 3, false), AGB_MF(subsurface, 1, false),
    AGB_MF(subsurface_color, 3, false), AGB_MF(subsurface_radius, 3, false),
    AGB_MF(subsurface_scale, 1, false), AGB_MF(subsurface_anisotropy, 1, false), AGB_MF(sheen, 1, false),
    AGB_MF(sheen_color, 3, false), AGB_MF(sheen_roughness, 1, false), AGB_MF(coat, 1, false),
    AGB_MF(coat_color, 3, false), AGB_MF(coat_roughness, 1, false), AGB_MF(coat_anisotropy, 1, false),
    AGB_MF(coat_rotation, 1, false), AGB_MF(coat_IOR, 1, false), AGB_MF(coat_affect_color, 1, false),
    AGB_MF(coat_affect_roughness, 1, false), AGB_MF(emission, 1, false), AGB_MF(emission_color, 3, false),
    AGB_MF(opacity, 3, false), AGB_MF(thin_walled, 1, true),
    // Texture transforms (MaterialBase.cpp:61-86).
    AGB_MF(base_color_image_offset, 2, false), AGB_MF(base_color_image_scale, 2, false),
    AGB_MF(base_color_image_pivot, 2, false), AGB_MF(base_color_image_rotation, 1, false),
    AGB_MF(specular_roughness_image_offset, 2, false), AGB_MF(specular_roughness_image_scale, 2, false),
    AGB_MF(specular_roughness_image_pivot, 2, false), AGB_MF(specular_roughness_image_rotation, 1, false),
    AGB_MF(emission_color_image_offset, 2, false), AGB_MF(emission_color_image_scale, 2, false),
    AGB_MF(emission_color_image_pivot, 2, false), AGB_MF(emission_color_image_rotation, 1, false),
    AGB_MF(opacity_image_offset, 2, false), AGB_MF(opacity_image_scale, 2, false),
    AGB_MF(opacity_image_pivot, 2, false), AGB_MF(opacity_image_rotation, 1, false),
    AGB_MF(normal_image_offset, 2, false), AGB_MF(normal_image_scale, 2, false),
    AGB_MF(normal_image_pivot, 2, false), AGB_MF(normal_image_rotation, 1, false),
};
// Texture properties (MaterialBase.cpp:91-95, 199-213): the image path, its texture slot and the
// material block's has_<name> flag, set when the texture is present.
struct TexField
{
    const char* name;
    int slot;
    size_t hasOffset;
};
#define AGB_TF(field, slot) { #field, slot, offsetof(agb_material, has_##field) }
const TexField kTexFields[] = {
    AGB_TF(base_color_image, AGB_TEX_BASE_COLOR), AGB_TF(specular_roughness_image, AGB_TEX_SPECULAR_ROUGHNESS),
    AGB_TF(opacity_image, AGB_TEX_OPACITY), AGB_TF(normal_image, AGB_TEX_NORMAL),
    AGB_TF(emission_color_image, AGB_TEX_EMISSION),
};
#undef AGB_TF
#undef AGB_MF

// Built-in Standard Surface defaults (MaterialBase.cpp:109-167).
agb_material defaultMaterial()
{
    agb_material m;
    std::memset(&m, 0, sizeof m);
    auto set3 = [](float* d, float a, float b, float c) { d[0] = a; d[1] = b; d[2] = c; };
    m.base = 0.8f;
    set3(m.base_color, 1, 1, 1);
    m.specular = 1.f;
    set3(m.specular_color, 1, 1, 1);
    m.specular_roughness = 0.2f;
    m.specular_IOR       = 1.5f;
    set3(m.transmission_color, 1, 1, 1);
    set3(m.subsurface_color, 1, 1, 1);
    set3(m.subsurface_radius, 1, 1, 1);
    m.subsurface_scale = 1.f;
    set3(m.sheen_color, 1, 1, 1);
    m.sheen_roughness = 0.3f;
    set3(m.coat_color, 1, 1, 1);
    m.coat_roughness = 0.1f;
    m.coat_IOR       = 1.5f;
    set3(m.emission_color, 1, 1, 1);
    set3(m.opacity, 1, 1, 1);
    for (float* s : { m.base_color_image_scale, m.specular_roughness_image_scale, m.emission_color_image_scale,
             m.opacity_image_scale, m.normal_image_scale })
        s[0] = s[1] = 1.f;
    return m;
}

class Scene : public IScene
{
public:
    explicit Scene(std::shared_ptr<LoadResourceFunction> l) : loader(std::move(l)) {}
    std::shared_ptr<LoadResourceFunction> loader; // the renderer's; an empty function reads files
    struct Geometry
    {
        GeometryDescriptor desc;
        int32_t handle = -1;
        float bounds[6] = { 1e30f, 1e30f, 1e30f, -1e30f, -1e30f, -1e30f };
    };
    struct Image
    {
        ImageDescriptor desc;
        int32_t handle    = -1; // environment use: nearest filtering
        int32_t texHandle[2] = { -1, -1 }; // material textures: nearest, bilinear filtering
    };
    struct Instance
    {
        Path geometry;
        Properties props;
    };

    std::map<Path, Geometry> geometries;
    std::map<Path, Image> images;
    std::map<Path, Properties> materials;
    std::map<Path, Properties> environments;
    std::map<Path, Properties> samplers;
    // Per material: texture properties fed by MaterialX image nodes (sampled bilinearly).
    std::map<Path, std::set<std::string>> materialXBilinear;
    std::vector<std::pair<Path, Instance>> instances; // insertion order
    std::vector<std::shared_ptr<Light>> lights;
    std::shared_ptr<GroundPlane> groundPlane; // null: the default, disabled plane
    Path environment;
    bool hasBounds = false;
    vec3 bmin{}, bmax{};
    bool dirty     = true;
    agb_context* ctx = nullptr; // the context the scene was last activated on

    void setGeometryDescriptor(const Path& p, const GeometryDescriptor& d) override
    {
        if (d.type != PrimitiveType::Triangles || !d.getAttributeData || d.vertexDesc.count == 0)
            throw Error("setGeometryDescriptor: triangle geometry with vertices and a data callback required");
        if (!d.vertexDesc.attributes.count(Names::VertexAttributes::kPosition) ||
            d.vertexDesc.attributes.at(Names::VertexAttributes::kPosition) != AttributeFormat::Float3)
            throw Error("setGeometryDescriptor: positions must be Float3");
        geometries[p] = Geometry{ d, -1 };
        dirty         = true;
    }
    void setImageDescriptor(const Path& p, const ImageDescriptor& d) override
    {
        if (!d.getData)
            throw Error("setImageDescriptor: a data callback is required");
        images[p] = Image{ d };
        dirty     = true;
    }
    // The file is read when the image is first used and released once uploaded (the scene keeps
    // the path, so a context change reads it again).
    void setImageFromFilePath(const Path& p, const std::string& filePath, bool linearize, bool) override
    {
        struct FileImage
        {
            std::vector<uint8_t> rgba8;
            std::vector<float> rgb32;
            int w = 0, h = 0;
        };
        const std::string file = filePath.empty() ? p : filePath;
        auto store             = std::make_shared<FileImage>();
        ImageDescriptor d;
        d.linearize = linearize;
        auto isHDR  = [](const std::string& f) {
            return f.size() >= 4 && (f.compare(f.size() - 4, 4, ".hdr") == 0 || f.compare(f.size() - 4, 4, ".HDR") == 0);
        };
        d.getData = [file, store, isHDR, loader = loader](ImageData& out) {
            bool hdr = isHDR(file);
            if (store->rgba8.empty() && store->rgb32.empty())
            {
                std::string err;
                bool ok;
                if (*loader)
                {
                    std::vector<unsigned char> bytes;
                    std::string name = file;
                    ok = (*loader)(file, &bytes, &name);
                    if (!ok)
                        err = "the resource loader failed";
                    else
                    {
                        hdr = isHDR(name);
                        std::string data(bytes.begin(), bytes.end());
                        ok  = hdr ? decodeHDR(data, store->rgb32, store->w, store->h, err)
                                  : decodePNG(data, store->rgba8, store->w, store->h, err);
                    }
                }
                else
                    ok = hdr ? loadHDRFile(file, store->rgb32, store->w, store->h, err)
                             : loadPNGFile(file, store->rgba8, store->w, store->h, err);
                if (!ok)
                {
                    logError("image " + file + ": " + err);
                    return false;
                }
            }
            out.dimensions = { store->w, store->h };
            if (!store->rgb32.empty())
            {
                out.pPixelBuffer = store->rgb32.data();
                out.bytesPerRow  = size_t(store->w) * 12;
                out.bufferSize   = store->rgb32.size() * 4;
                out.format       = ImageFormat::Float_RGB;
            }
            else
            {
                out.pPixelBuffer = store->rgba8.data();
                out.bytesPerRow  = size_t(store->w) * 4;
                out.bufferSize   = store->rgba8.size();
                out.format       = ImageFormat::Integer_RGBA;
            }
            return true;
        };
        d.updateComplete = [store](const ImageData&) {
            std::vector<uint8_t>().swap(store->rgba8);
            std::vector<float>().swap(store->rgb32);
        };
        images[p] = Image{ d }; // both texture handles start unset (-1)
        dirty     = true;
    }
    void setMaterialType(const Path& p, const std::string& type, const std::string& document) override
    {
        Properties& m = materials[p];
        if (type == Names::MaterialTypes::kMaterialX || type == Names::MaterialTypes::kMaterialXPath)
        {
            // The document's standard_surface constants become the material's values; properties
            // set afterwards override them.
            Properties fromDoc;
            std::string warnings;
            std::vector<MaterialXImage> imgs;
            bool ok = type == Names::MaterialTypes::kMaterialX
                ? materialXToProperties(document, "", fromDoc, warnings, imgs)
                : materialXFileToProperties(document, fromDoc, warnings, &imgs);
            if (!warnings.empty())
                logError("setMaterialType " + p + ": " + warnings);
            if (ok)
            {
                // MaterialX image nodes filter linearly (their filtertype default).  The slots are
                // kept apart from the user's samplers, so no sampler name is taken; their address
                // modes (uaddressmode / vaddressmode) are not read: the device wraps.
                std::set<std::string>& lin = materialXBilinear[p];
                lin.clear();
                for (const MaterialXImage& im : imgs)
                {
                    setImageFromFilePath(im.image, im.file, im.linearize, false);
                    lin.insert(im.property);
                }
                merge(m, fromDoc);
            }
        }
        else if (type != Names::MaterialTypes::kBuiltIn)
            logError("setMaterialType: unknown material type " + type + "; " + p +
                " uses the built-in Standard Surface material");
        dirty = true;
    }
    void setSamplerProperties(const Path& p, const Properties& props) override
    {
        merge(samplers[p], props);
        dirty = true;
    }
    void setMaterialProperties(const Path& p, const Properties& props) override
    {
        merge(materials[p], props);
        dirty = true;
    }
    bool addInstance(const Path& p, const Path& geometry, const Properties& props) override
    {
        for (auto& kv : instances)
            if (kv.first == p)
            {
                logError("addInstance: " + p + " already exists");
                return false;
            }
        instances.push_back({ p, Instance{ geometry, props } });
        dirty = true;
        return true;
    }
    void setInstanceProperties(const Path& p, const Properties& props) override
    {
        for (auto& kv : instances)
            if (kv.first == p)
            {
                merge(kv.second.props, props);
                dirty = true;
                return;
            }
        logError("setInstanceProperties: no instance " + p);
    }
    void removeInstance(const Path& p) override
    {
        instances.erase(std::remove_if(instances.begin(), instances.end(),
                            [&](const std::pair<Path, Instance>& kv) { return kv.first == p; }),
            instances.end());
        dirty = true;
    }
    bool setEnvironmentProperties(const Path& p, const Properties& props) override
    {
        merge(environments[p], props);
        dirty = true;
        return true;
    }
    bool setEnvironment(const Path& p) override
    {
        environment = p;
        dirty       = true;
        return true;
    }
    void setBounds(const vec3& mn, const vec3& mx) override
    {
        bmin      = mn;
        bmax      = mx;
        hasBounds = true;
    }
    void setGroundPlanePointer(const IGroundPlanePtr& g) override
    {
        groundPlane = std::dynamic_pointer_cast<GroundPlane>(g);
        if (g && !groundPlane)
            throw Error("setGroundPlanePointer: not a ground plane of this renderer");
    }
    // The ground plane's current values, read at every render as the reference's
    // PTGroundPlane::update does (PTScene.cpp:779).
    void applyGroundPlane()
    {
        if (!groundPlane)
        {
            check(agb_ground_plane_set(ctx, nullptr), "ground plane");
            return;
        }
        agb_ground_plane g = groundPlane->data();
        check(agb_ground_plane_set(ctx, &g), "ground plane");
    }
    ILightPtr addLightPointer(const std::string& type) override
    {
        if (type != Names::LightTypes::kDistantLight)
            throw Error("addLightPointer: only " + Names::LightTypes::kDistantLight + " is supported");
        auto l = std::make_shared<Light>();
        lights.push_back(l);
        return l;
    }

    // Uploads what changed to ctx (a new context re-uploads everything).
    void activate(agb_context* c)
    {
        if (c != ctx)
        {
            for (auto& g : geometries)
                g.second.handle = -1;
            for (auto& i : images)
                i.second.handle = i.second.texHandle[0] = i.second.texHandle[1] = -1;
            ctx   = c;
            dirty = true;
        }
        if (!dirty)
            return;
        // Geometry referenced by instances, pulled once.
        for (auto& kv : instances)
        {
            auto it = geometries.find(kv.second.geometry);
            if (it == geometries.end())
                throw Error("render: instance " + kv.first + " refers to unknown geometry " + kv.second.geometry);
            if (it->second.handle < 0)
                pullGeometry(it->first, it->second);
        }
        std::vector<agb_material> mats(1, defaultMaterial());
        std::vector<agb_material_textures> texs(1);
        std::map<Path, int32_t> matIndex;
        bool anyTexture = false;
        // Node-graph programs of MaterialX materials, gathered into one operation / constant table.
        std::vector<int32_t> graphFirst(1, 0), graphCount(1, 0);
        std::vector<agb_graph_op> graphOps;
        std::vector<float> graphConsts;
        for (auto& kv : materials)
        {
            agb_material m = defaultMaterial();
            agb_material_textures t;
            for (int k = 0; k < AGB_TEX_SLOTS; k++)
                t.image[k] = -1;
            int32_t gFirst = int32_t(graphOps.size()), gCount = 0;
            for (auto& p : kv.second)
            {
                if (p.first == "materialx_graph")
                {
                    if (auto* prog = std::get_if<Strings>(&p.second))
                        gCount = appendGraph(*prog, kv.first, graphOps, graphConsts);
                    continue;
                }
                if (applyTextureProperty(m, t, p.first, p.second, kv.first, kv.second))
                    continue;
                applyMaterialProperty(m, p.first, p.second, kv.first);
            }
            graphFirst.push_back(gCount ? gFirst : 0);
            graphCount.push_back(gCount);
            for (int k = 0; k < AGB_TEX_SLOTS; k++)
                anyTexture = anyTexture || t.image[k] >= 0;
            matIndex[kv.first] = int32_t(mats.size());
            mats.push_back(m);
            texs.push_back(t);
        }
        for (int k = 0; k < AGB_TEX_SLOTS; k++)
            texs[0].image[k] = -1;
        check(agb_materials_set(ctx, mats.data(), anyTexture ? texs.data() : nullptr, uint32_t(mats.size())),
            "upload materials");
        if (!graphOps.empty())
            check(agb_material_graphs_set(ctx, graphFirst.data(), graphCount.data(), uint32_t(mats.size()),
                      graphOps.data(), uint32_t(graphOps.size()), graphConsts.data(), uint32_t(graphConsts.size() / 4)),
                "upload material graphs");
        std::vector<agb_instance> insts;
        for (auto& kv : instances)
        {
            const Properties& p = kv.second.props;
            if (auto* vis = find<bool>(p, Names::InstanceProperties::kVisible))
                if (!*vis)
                    continue;
            agb_instance in;
            std::memset(&in, 0, sizeof in);
            in.geometry = geometries[kv.second.geometry].handle;
            in.material = 0;
            if (auto* mp = find<std::string>(p, Names::InstanceProperties::kMaterial))
            {
                auto it = matIndex.find(*mp);
                if (it == matIndex.end())
                    logError("instance " + kv.first + ": unknown material " + *mp + ", using the default");
                else
                    in.material = it->second;
            }
            const mat4* t = find<mat4>(p, Names::InstanceProperties::kTransform);
            rows3x4(t ? *t : kIdentity, in.object_to_world);
            // Material layers (Resources.cpp:318-335; PTScene.cpp:1051-1166): layer i is the
            // material of layer_materials[i] with the texture coordinates of the geometry
            // layer_geometry[i], one per vertex of the instance's geometry.
            const Strings* lm = find<Strings>(p, Names::InstanceProperties::kMaterialLayers);
            const Strings* lg = find<Strings>(p, Names::InstanceProperties::kGeometryLayers);
            if (lm && !lm->empty())
            {
                layerSets.emplace_back();
                std::vector<agb_layer>& ls = layerSets.back();
                const Geometry& base       = geometries[kv.second.geometry];
                for (size_t li = 0; li < lm->size(); li++)
                {
                    auto mit = matIndex.find((*lm)[li]);
                    if (mit == matIndex.end())
                    {
                        logError("instance " + kv.first + ": unknown layer material " + (*lm)[li]);
                        continue;
                    }
                    if (!lg || li >= lg->size())
                    {
                        logError("instance " + kv.first + ": layer " + std::to_string(li) + " has no geometry");
                        continue;
                    }
                    const std::vector<float>* uv = layerTexcoords((*lg)[li], base.desc.vertexDesc.count);
                    if (!uv)
                    {
                        logError("instance " + kv.first + ": layer geometry " + (*lg)[li] +
                            " needs texture coordinates for every vertex of " + kv.second.geometry);
                        continue;
                    }
                    agb_layer l{};
                    l.material  = mit->second;
                    l.texcoords = uv->data();
                    ls.push_back(l);
                }
                in.layer_count = int32_t(ls.size());
                in.layers      = ls.empty() ? nullptr : ls.data();
            }
            insts.push_back(in);
        }
        check(agb_instances_set(ctx, insts.data(), uint32_t(insts.size())), "upload instances");
        layerSets.clear();
        layerUVs.clear();
        applyEnvironment();
        dirty = false;
    }

    void pullGeometry(const Path& path, Geometry& g)
    {
        const GeometryDescriptor& d = g.desc;
        size_t nv = d.vertexDesc.count, ni = d.indexCount;
        AttributeDataMap buffers;
        for (auto& a : d.vertexDesc.attributes)
            buffers[a.first] = AttributeData{};
        if (ni)
            buffers[Names::VertexAttributes::kIndices] = AttributeData{};
        if (!d.getAttributeData(buffers, 0, nv, 0, ni))
            throw Error("geometry " + path + ": getAttributeData failed");
        auto gather = [&](const std::string& name, int comps) -> std::vector<float> {
            std::vector<float> out;
            auto it = buffers.find(name);
            if (it == buffers.end() || !it->second.address)
                return out;
            const AttributeData& a = it->second;
            size_t stride = a.stride ? a.stride : comps * sizeof(float);
            out.resize(nv * comps);
            for (size_t v = 0; v < nv; v++)
                std::memcpy(&out[v * comps], static_cast<const uint8_t*>(a.address) + a.offset + v * stride,
                    comps * sizeof(float));
            return out;
        };
        std::vector<float> pos = gather(Names::VertexAttributes::kPosition, 3);
        if (pos.empty())
            throw Error("geometry " + path + ": no positions");
        std::vector<float> nrm = gather(Names::VertexAttributes::kNormal, 3);
        std::vector<float> uv  = gather(Names::VertexAttributes::kTexCoord0, 2);
        std::vector<uint32_t> idx;
        if (ni)
        {
            const AttributeData& a = buffers[Names::VertexAttributes::kIndices];
            if (!a.address)
                throw Error("geometry " + path + ": no indices");
            idx.resize(ni);
            size_t stride = a.stride ? a.stride : sizeof(uint32_t);
            for (size_t k = 0; k < ni; k++)
                std::memcpy(&idx[k], static_cast<const uint8_t*>(a.address) + a.offset + k * stride, 4);
        }
        if (d.attributeUpdateComplete)
            d.attributeUpdateComplete(buffers, 0, nv, 0, ni);
        check(agb_geometry_create(ctx, pos.data(), nrm.empty() ? nullptr : nrm.data(),
                  uv.empty() ? nullptr : uv.data(), idx.empty() ? nullptr : idx.data(), uint32_t(nv),
                  uint32_t(ni ? ni : nv), &g.handle),
            "geometry " + path);
        for (size_t v = 0; v < nv; v++)
            for (int k = 0; k < 3; k++)
            {
                g.bounds[k]     = std::min(g.bounds[k], pos[3 * v + k]);
                g.bounds[3 + k] = std::max(g.bounds[3 + k], pos[3 * v + k]);
            }
    }

    int32_t imageHandle(const Path& path)
    {
        auto it = images.find(path);
        if (it == images.end())
            throw Error("unknown image " + path);
        Image& im = it->second;
        if (im.handle >= 0)
            return im.handle;
        ImageData data;
        if (!im.desc.getData(data) || !data.pPixelBuffer)
            throw Error("image " + path + ": getData failed");
        int32_t fmt = data.format == ImageFormat::Integer_RGBA ? AGB_FORMAT_RGBA8_UNORM
            : data.format == ImageFormat::Float_RGBA           ? AGB_FORMAT_RGBA32F
                                                               : AGB_FORMAT_RGB32F;
        check(agb_image_create(ctx, data.pPixelBuffer, uint32_t(data.dimensions[0]), uint32_t(data.dimensions[1]),
                  fmt, 0, &im.handle),
            "image " + path);
        if (im.desc.updateComplete)
            im.desc.updateComplete(data);
        return im.handle;
    }

    // Layer arrays and layer texture coordinates of the activation in progress.
    std::list<std::vector<agb_layer>> layerSets;
    std::map<Path, std::vector<float>> layerUVs;

    // The texture coordinates of a layer geometry, pulled from its descriptor; null unless it
    // has one pair per vertex of a geometry with `vertexCount` vertices.
    const std::vector<float>* layerTexcoords(const Path& path, size_t vertexCount)
    {
        auto cached = layerUVs.find(path);
        if (cached != layerUVs.end())
            return cached->second.size() == vertexCount * 2 ? &cached->second : nullptr;
        std::vector<float>& uv = layerUVs[path];
        auto it = geometries.find(path);
        if (it == geometries.end())
            return nullptr;
        const GeometryDescriptor& d = it->second.desc;
        if (!d.vertexDesc.attributes.count(Names::VertexAttributes::kTexCoord0) || d.vertexDesc.count != vertexCount)
            return nullptr;
        AttributeDataMap buffers;
        buffers[Names::VertexAttributes::kTexCoord0] = AttributeData{};
        if (!d.getAttributeData(buffers, 0, d.vertexDesc.count, 0, 0))
            return nullptr;
        const AttributeData& a = buffers[Names::VertexAttributes::kTexCoord0];
        if (a.address)
        {
            size_t stride = a.stride ? a.stride : 2 * sizeof(float);
            uv.resize(vertexCount * 2);
            for (size_t v = 0; v < vertexCount; v++)
                std::memcpy(&uv[v * 2], static_cast<const uint8_t*>(a.address) + a.offset + v * stride,
                    2 * sizeof(float));
        }
        if (d.attributeUpdateComplete)
            d.attributeUpdateComplete(buffers, 0, d.vertexDesc.count, 0, 0);
        return uv.size() == vertexCount * 2 ? &uv : nullptr;
    }

    // A material texture: nearest filtering with the renderer's default sampler
    // (HGIRenderer.cpp:108-112, HgiSamplerDesc's default filters), bilinear with a sampler of the
    // material's own (HGISampler.cpp:21-41; HGIScene.cpp:249-251, 512); an 8-bit image with
    // `linearize` set is decoded from sRGB to linear values first, as an sRGB texture format
    // decodes it.
    // Appends a MaterialX material's node-graph program (the `materialx_graph` property: "op",
    // "const" and "image" lines, indices local to the program) to the scene's tables, constant and
    // image indices rebased; returns its operation count (0 when it cannot be read).
    int32_t appendGraph(const Strings& prog, const Path& material, std::vector<agb_graph_op>& ops,
        std::vector<float>& consts)
    {
        std::vector<agb_graph_op> local;
        std::vector<float> k;
        std::vector<int32_t> imageHandles;
        try
        {
            for (const std::string& line : prog)
            {
                if (line.compare(0, 3, "op ") == 0)
                {
                    int v[7];
                    if (std::sscanf(line.c_str() + 3, "%d %d %d %d %d %d %d", &v[0], &v[1], &v[2], &v[3], &v[4], &v[5],
                            &v[6]) != 7)
                        throw Error("bad operation '" + line + "'");
                    agb_graph_op o;
                    o.op  = uint8_t(v[0]);
                    o.dst = uint8_t(v[1]);
                    o.a   = uint8_t(v[2]);
                    o.b   = uint8_t(v[3]);
                    o.c   = uint8_t(v[4]);
                    o.d   = uint8_t(v[5]);
                    o.imm = uint16_t(v[6]);
                    local.push_back(o);
                }
                else if (line.compare(0, 6, "const ") == 0)
                {
                    float f[4];
                    if (std::sscanf(line.c_str() + 6, "%g %g %g %g", &f[0], &f[1], &f[2], &f[3]) != 4)
                        throw Error("bad constant '" + line + "'");
                    k.insert(k.end(), f, f + 4);
                }
                else if (line.compare(0, 6, "image ") == 0)
                {
                    std::string path   = line.substr(6);
                    const bool nearest = path.size() > 8 && path.compare(path.size() - 8, 8, ":nearest") == 0;
                    if (nearest)
                        path.resize(path.size() - 8);
                    imageHandles.push_back(textureHandle(path, !nearest));
                }
            }
        }
        catch (const Error& e)
        {
            logError("material " + material + ": node graph not used: " + e.what());
            return 0;
        }
        const uint16_t kBase = uint16_t(consts.size() / 4);
        for (agb_graph_op o : local)
        {
            if (o.op == AGB_GOP_CONST)
                o.imm = uint16_t(o.imm + kBase);
            else if (o.op == AGB_GOP_IMAGE)
                o.imm = o.imm < imageHandles.size() ? uint16_t(imageHandles[o.imm]) : uint16_t(0xFFFF);
            ops.push_back(o);
        }
        consts.insert(consts.end(), k.begin(), k.end());
        return int32_t(local.size());
    }

    int32_t textureHandle(const Path& path, bool bilinear)
    {
        auto it = images.find(path);
        if (it == images.end())
            throw Error("unknown image " + path);
        Image& im       = it->second;
        int32_t& handle = im.texHandle[bilinear ? 1 : 0];
        if (handle >= 0)
            return handle;
        ImageData data;
        if (!im.desc.getData(data) || !data.pPixelBuffer)
            throw Error("image " + path + ": getData failed");
        const uint32_t w = uint32_t(data.dimensions[0]), h = uint32_t(data.dimensions[1]);
        const bool linearize = data.overrideLinearize ? data.linearize : im.desc.linearize;
        if (data.format == ImageFormat::Integer_RGBA && linearize)
        {
            std::vector<float> px(size_t(w) * h * 4);
            size_t row = data.bytesPerRow ? data.bytesPerRow : size_t(w) * 4;
            for (uint32_t y = 0; y < h; y++)
                for (uint32_t x = 0; x < w; x++)
                {
                    const uint8_t* s8 = static_cast<const uint8_t*>(data.pPixelBuffer) + y * row + x * 4;
                    float* d          = &px[(size_t(y) * w + x) * 4];
                    for (int c = 0; c < 3; c++)
                    {
                        double v = double(s8[c]) / 255.0;
                        d[c] = float(v <= 0.04045 ? v / 12.92 : std::pow((v + 0.055) / 1.055, 2.4));
                    }
                    d[3] = float(s8[3]) / 255.f;
                }
            check(agb_image_create(ctx, px.data(), w, h, AGB_FORMAT_RGBA32F, bilinear ? 1 : 0, &handle),
                "image " + path);
        }
        else
        {
            int32_t fmt = data.format == ImageFormat::Integer_RGBA ? AGB_FORMAT_RGBA8_UNORM
                : data.format == ImageFormat::Float_RGBA           ? AGB_FORMAT_RGBA32F
                                                                   : AGB_FORMAT_RGB32F;
            check(agb_image_create(ctx, data.pPixelBuffer, w, h, fmt, bilinear ? 1 : 0, &handle), "image " + path);
        }
        if (im.desc.updateComplete)
            im.desc.updateComplete(data);
        return handle;
    }

    // Texture image and sampler properties; false for any other property.
    bool applyTextureProperty(agb_material& m, agb_material_textures& t, const std::string& name,
        const PropertyValue& v, const Path& path, const Properties& all)
    {
        for (const TexField& f : kTexFields)
        {
            if (name == f.name)
            {
                auto* ip = std::get_if<std::string>(&v);
                if (!ip)
                {
                    logError("material " + path + ": " + name + " wants an image path");
                    return true;
                }
                int32_t has = 0;
                if (!ip->empty())
                {
                    const std::string* sampler = find<std::string>(all, std::string(f.name) + "_sampler");
                    bool bilinear = sampler && !sampler->empty() && samplers.count(*sampler);
                    auto mx       = materialXBilinear.find(path);
                    if (mx != materialXBilinear.end() && mx->second.count(f.name))
                        bilinear = true;
                    t.image[f.slot] = textureHandle(*ip, bilinear);
                    has             = 1;
                }
                std::memcpy(reinterpret_cast<uint8_t*>(&m) + f.hasOffset, &has, 4);
                return true;
            }
            if (name == std::string(f.name) + "_sampler")
            {
                auto* sp = std::get_if<std::string>(&v);
                if (sp && !sp->empty())
                {
                    auto it = samplers.find(*sp);
                    if (it == samplers.end())
                        logError("material " + path + ": unknown sampler " + *sp);
                    else
                        for (const std::string& k :
                            { Names::SamplerProperties::kAddressModeU, Names::SamplerProperties::kAddressModeV })
                            if (auto* mode = find<std::string>(it->second, k))
                                if (*mode != Names::AddressModes::kWrap)
                                    logError("sampler " + *sp + ": address mode " + *mode +
                                        " is sampled with wrapping");
                }
                return true;
            }
        }
        return false;
    }

    void applyEnvironment()
    {
        agb_environment_data e;
        std::memset(&e, 0, sizeof e);
        // Defaults (EnvironmentBase.cpp:33-45).
        const Properties empty;
        const Properties& p = environments.count(environment) ? environments[environment] : empty;
        auto v3 = [&](const std::string& n, vec3 def, float* out) {
            auto* v = find<vec3>(p, n);
            vec3 x  = v ? *v : def;
            out[0] = x[0];
            out[1] = x[1];
            out[2] = x[2];
        };
        v3(Names::EnvironmentProperties::kLightTop, { 1, 1, 1 }, e.light_top);
        v3(Names::EnvironmentProperties::kLightBottom, { 0, 0, 0 }, e.light_bottom);
        v3(Names::EnvironmentProperties::kBackgroundTop, { 0.02f, 0.25f, 0.60f }, e.background_top);
        v3(Names::EnvironmentProperties::kBackgroundBottom, { 0.32f, 0.79f, 1.0f }, e.background_bottom);
        const mat4* lt = find<mat4>(p, Names::EnvironmentProperties::kLightTransform);
        mat4 lm        = lt ? *lt : kIdentity, lmi;
        if (!inverse4(lm, lmi))
            throw Error("environment: light transform is singular");
        rowMajor(lm, e.light_transform);
        rowMajor(lmi, e.light_transform_inv);
        const mat4* bt = find<mat4>(p, Names::EnvironmentProperties::kBackgroundTransform);
        rowMajor(bt ? *bt : kIdentity, e.background_transform);
        if (auto* b = find<bool>(p, Names::EnvironmentProperties::kBackgroundUseScreen))
            e.background_use_screen = *b ? 1 : 0;
        int32_t light = -1, background = -1;
        if (auto* li = find<std::string>(p, Names::EnvironmentProperties::kLightImage))
            if (!li->empty())
                light = imageHandle(*li);
        if (auto* bi = find<std::string>(p, Names::EnvironmentProperties::kBackgroundImage))
            if (!bi->empty())
                background = imageHandle(*bi);
        check(agb_environment_set(ctx, &e, light, background), "environment");
    }

    static void applyMaterialProperty(agb_material& m, const std::string& name, const PropertyValue& v,
        const Path& path)
    {
        for (const MatField& f : kMatFields)
        {
            if (name != f.name)
                continue;
            float* dst = reinterpret_cast<float*>(reinterpret_cast<uint8_t*>(&m) + f.offset);
            if (f.integer)
            {
                int32_t iv = 0;
                if (auto* b = std::get_if<bool>(&v))
                    iv = *b;
                else if (auto* i = std::get_if<int>(&v))
                    iv = *i;
                else
                {
                    logError("material " + path + ": " + name + " wants a boolean");
                    return;
                }
                std::memcpy(dst, &iv, 4);
                return;
            }
            if (f.count == 3)
            {
                if (auto* x = std::get_if<vec3>(&v))
                {
                    dst[0] = (*x)[0];
                    dst[1] = (*x)[1];
                    dst[2] = (*x)[2];
                    return;
                }
            }
            else if (f.count == 2)
            {
                if (auto* x = std::get_if<vec2>(&v))
                {
                    dst[0] = (*x)[0];
                    dst[1] = (*x)[1];
                    return;
                }
            }
            else if (auto* x = std::get_if<float>(&v))
            {
                dst[0] = *x;
                return;
            }
            logError("material " + path + ": " + name + " has the wrong type");
            return;
        }
        logError("material " + path + ": unknown property " + name);
    }

    void bounds(float out[6]) const
    {
        if (hasBounds)
        {
            for (int k = 0; k < 3; k++)
            {
                out[k]     = bmin[k];
                out[3 + k] = bmax[k];
            }
            return;
        }
        for (int k = 0; k < 3; k++)
        {
            out[k]     = 1e30f;
            out[3 + k] = -1e30f;
        }
        for (auto& kv : instances)
        {
            auto it = geometries.find(kv.second.geometry);
            if (it == geometries.end() || it->second.handle < 0)
                continue;
            const mat4* t = find<mat4>(kv.second.props, Names::InstanceProperties::kTransform);
            const mat4& m = t ? *t : kIdentity;
            const float* b = it->second.bounds;
            for (int c = 0; c < 8; c++)
            {
                float pt[3] = { b[(c & 1) ? 3 : 0], b[(c & 2) ? 4 : 1], b[(c & 4) ? 5 : 2] };
                for (int r = 0; r < 3; r++)
                {
                    float w = m[r] * pt[0] + m[4 + r] * pt[1] + m[8 + r] * pt[2] + m[12 + r];
                    out[r]     = std::min(out[r], w);
                    out[3 + r] = std::max(out[3 + r], w);
                }
            }
        }
    }
};

class Renderer : public IRenderer
{
public:
    agb_context* ctx = nullptr;
    std::shared_ptr<Scene> scene;
    TargetAssignments targets;
    Values opts;
    mat4 view = kIdentity, proj = kIdentity;
    float focalDistance = 1.f, lensRadius = 0.f;

    explicit Renderer(agb_context* c) : ctx(c)
    {
        // Option defaults (RendererBase.cpp:59-89).
        opts.setFloat("maxLuminance", 1000.f);
        opts.setInt("traceDepth", 5);
        opts.setBoolean("isToneMappingEnabled", false);
        opts.setBoolean("isGammaCorrectionEnabled", true);
        opts.setFloat3("brightness", { 1.f, 1.f, 1.f });
        opts.setBoolean("isRussianRouletteEnabled", true);
        opts.setInt("russianRouletteStartDepth", 3);
        opts.setBoolean("isDiffuseOnlyEnabled", false);
        // The HGI backend forces opaque shadows (HGIRenderer.cpp:491); false selects the
        // transparent (any-hit opacity) shadows of the DirectX backend.
        opts.setBoolean("isForceOpaqueShadowsEnabled", true);
    }
    ~Renderer() override
    {
        if (ctx)
            agb_context_destroy(ctx);
    }
    std::shared_ptr<LoadResourceFunction> loader = std::make_shared<LoadResourceFunction>();
    IScenePtr createScene() override { return std::make_shared<Scene>(loader); }
    void setLoadResourceFunction(LoadResourceFunction func) override { *loader = std::move(func); }
    IGroundPlanePtr createGroundPlanePointer() override { return std::make_shared<GroundPlane>(); }
    void setScene(const IScenePtr& s) override
    {
        scene = std::dynamic_pointer_cast<Scene>(s);
        if (s && !scene)
            throw Error("setScene: the scene was not created by this renderer");
    }
    IRenderBufferPtr createRenderBuffer(int w, int h, ImageFormat f) override
    {
        if (w <= 0 || h <= 0 || f == ImageFormat::Float_RGB)
            throw Error("createRenderBuffer: positive size, Integer_RGBA or Float_RGBA");
        return std::make_shared<RenderBuffer>(w, h, f);
    }
    void setTargets(const TargetAssignments& t) override { targets = t; }
    void setOptions(const Properties& o) override
    {
        merge(opts.props, o);
    }
    IValues& options() override { return opts; }
    void setCamera(const mat4& v, const mat4& p, float fd, float lr) override
    {
        view          = v;
        proj          = p;
        focalDistance = fd;
        lensRadius    = lr;
    }

    // RendererBase::updateFrameDataGPUStruct (RendererBase.cpp:225-295) for the current options.
    agb_frame_data frameData(uint32_t W, uint32_t H) const
    {
        agb_frame_data f;
        std::memset(&f, 0, sizeof f);
        // view-projection: proj * view (column-major).
        mat4 vp{};
        for (int r = 0; r < 4; r++)
            for (int c = 0; c < 4; c++)
            {
                double s = 0;
                for (int k = 0; k < 4; k++)
                    s += double(proj[4 * k + r]) * double(view[4 * c + k]);
                vp[4 * c + r] = float(s);
            }
        std::memcpy(f.camera_view_proj, vp.data(), 64);
        std::memcpy(f.camera_view_proj_prev, vp.data(), 64);
        mat4 inv;
        if (!inverse4(view, inv))
            throw Error("setCamera: view matrix is singular");
        rowMajor(inv, f.camera_inv_view);
        std::memcpy(f.camera_inv_view_prev, f.camera_inv_view, 64);
        f.view_size[0]        = float(2.0 / double(proj[0]));
        f.view_size[1]        = float(2.0 / double(proj[5]));
        f.is_ortho_projection = proj[15] == 1.f ? 1 : 0;
        f.focal_distance      = focalDistance;
        f.lens_radius         = lensRadius;
        f.time_delta_ms       = 1000.f / 60.f;
        float b[6];
        scene->bounds(b);
        bool valid = b[0] <= b[3];
        if (valid)
        {
            float dx = b[3] - b[0], dy = b[4] - b[1], dz = b[5] - b[2];
            f.scene_size = std::sqrt(dx * dx + dy * dy + dz * dz);
        }
        // Sky depth: twice the denoising range (RendererBase.cpp:206-224, :258).
        float range = 1.f;
        if (valid)
        {
            float zmin = 1e30f;
            for (int c = 0; c < 8; c++)
            {
                float pt[3] = { b[(c & 1) ? 3 : 0], b[(c & 2) ? 4 : 1], b[(c & 4) ? 5 : 2] };
                float z     = view[2] * pt[0] + view[6] * pt[1] + view[10] * pt[2] + view[14];
                zmin        = std::min(zmin, z);
            }
            range = std::min(std::max(-zmin * 1.1f, 1.f), 5.0e8f);
        }
        f.sky_view_z                      = -range * 2.f;
        f.is_force_opaque_shadows_enabled = opts.asBool("isForceOpaqueShadowsEnabled", true) ? 1 : 0;
        f.is_diffuse_only_enabled         = opts.asBool("isDiffuseOnlyEnabled", false) ? 1 : 0;
        f.trace_depth                     = std::max(1, std::min(10, opts.asInt("traceDepth", 5)));
        f.max_luminance                   = opts.asFloat("maxLuminance", 1000.f);
        f.is_russian_roulette_enabled     = opts.asBool("isRussianRouletteEnabled", true) ? 1 : 0;
        f.russian_roulette_start_depth    = std::max(0, opts.asInt("russianRouletteStartDepth", 3));
        // Distant lights (HGIScene.cpp:110-133): at most 4, direction negated.
        int n = int(std::min<size_t>(scene->lights.size(), 4));
        f.distant_light_count = n;
        for (int i = 0; i < n; i++)
        {
            const Values& v = scene->lights[i]->v;
            vec3 d = v.asFloat3(Names::LightProperties::kDirection, { 0, 0, -1 });
            vec3 c = v.asFloat3(Names::LightProperties::kColor, { 1, 1, 1 });
            f.distant_lights[i].cos_radius = std::cos(0.5f * v.asFloat(Names::LightProperties::kAngularDiameter, 0.1f));
            for (int k = 0; k < 3; k++)
            {
                f.distant_lights[i].direction[k]           = -d[k];
                f.distant_lights[i].color_and_intensity[k] = c[k];
            }
            f.distant_lights[i].color_and_intensity[3] = v.asFloat(Names::LightProperties::kIntensity, 1.f);
        }
        (void)W;
        (void)H;
        return f;
    }

    void render(uint32_t sampleStart, uint32_t sampleCount) override
    {
        if (!scene)
            throw Error("render: no scene");
        auto it = targets.find(AOV::Final);
        if (it == targets.end() || !it->second)
            throw Error("render: no Final target");
        auto* target = dynamic_cast<RenderBuffer*>(it->second.get());
        scene->activate(ctx);
        scene->applyGroundPlane();
        agb_frame_data f = frameData(uint32_t(target->w), uint32_t(target->h));
        check(agb_frame_set(ctx, &f), "render");
        agb_render_options o;
        std::memset(&o, 0, sizeof o);
        o.width        = uint32_t(target->w);
        o.height       = uint32_t(target->h);
        o.accumulation = AGB_ACCUM_RUNNING_MEAN;
        check(agb_render(ctx, &o, sampleStart, sampleCount, nullptr), "render");
        vec3 br = opts.asFloat3("brightness", { 1, 1, 1 });
        check(agb_post_process(ctx, AGB_ACCUM_RUNNING_MEAN, br.data(), opts.asBool("isToneMappingEnabled", false),
                  opts.asBool("isGammaCorrectionEnabled", true),
                  target->format == ImageFormat::Float_RGBA ? target->rgba32.data() : nullptr,
                  target->format == ImageFormat::Integer_RGBA ? target->rgba8.data() : nullptr),
            "render");
    }
    void waitForTask() override { check(agb_wait(ctx), "waitForTask"); }
    const std::vector<std::string>& builtInMaterials() override
    {
        static const std::vector<std::string> kNone;
        return kNone;
    }
};

} // namespace

void setLogCallback(std::function<void(const std::string&)> cb)
{
    std::lock_guard<std::mutex> g(g_logMutex);
    g_log = std::move(cb);
}

IRendererPtr createRenderer(IRenderer::Backend, uint32_t)
{
    agb_context* ctx = nullptr;
    if (agb_context_create(0, nullptr, &ctx) != AGB_OK)
    {
        logError(std::string("createRenderer: ") + agb_last_error());
        return nullptr;
    }
    return std::make_shared<Renderer>(ctx);
}

} // namespace agb_aurora
