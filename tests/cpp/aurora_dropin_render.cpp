// An Aurora client: renders a scene through Aurora's own public interface (<Aurora/Aurora.h>,
// namespace Aurora, glm types), obtaining the renderer from Aurora::createRenderer.  It compiles
// unchanged against the reference's header (Libraries/Aurora/API/Aurora/Aurora.h) and against this
// library's copy of that interface (include/Aurora/Aurora.h), and links against libagb_cuda.so.
//
// usage: aurora_dropin_render <scene file> <output file> [--pointers] [--late-materials] [--loader]
//   default: path-keyed resources (setGeometryDescriptor, setImageDescriptor,
//     setSamplerProperties, setMaterialType / setMaterialProperties, addInstance).
//   --pointers: renderer-owned objects instead (createGeometryPointer, createImagePointer,
//     createSamplerPointer, createMaterialPointer with IValues, addInstancePointer with layer
//     definitions).
//   --late-materials: one sample is rendered with the materials unset, then the materials are
//     set and the frame is rendered from sample 0.
//   --loader: image files (those MaterialX documents name) are read through a resource loader
//     installed with IRenderer::setLoadResourceFunction, which must be called.
// The scene file is the one tests/cpp/aurora_api_render.cpp reads (written by
// tests/test_aurora_api.py's write_scene); the output is u32 width, height, then f32 RGBA rows.
#include <Aurora/Aurora.h>
#include <glm/gtc/type_ptr.hpp>

#include <cstdio>
#include <cstring>
#include <functional>
#include <stdexcept>
#include <string>
#include <vector>

namespace A = Aurora;
namespace N = Aurora::Names;

namespace
{

struct Reader
{
    std::vector<uint8_t> buf;
    size_t pos = 0;
    template <class T>
    T get()
    {
        T v;
        if (pos + sizeof(T) > buf.size())
            throw std::runtime_error("scene file truncated");
        std::memcpy(&v, &buf[pos], sizeof(T));
        pos += sizeof(T);
        return v;
    }
    template <class T>
    std::vector<T> array(size_t n)
    {
        std::vector<T> v(n);
        if (pos + n * sizeof(T) > buf.size())
            throw std::runtime_error("scene file truncated");
        std::memcpy(v.data(), &buf[pos], n * sizeof(T));
        pos += n * sizeof(T);
        return v;
    }
    A::mat4 matrix()
    {
        auto v = array<float>(16);
        A::mat4 m;
        std::memcpy(glm::value_ptr(m), v.data(), sizeof(float) * 16); // column-major, as glm
        return m;
    }
    A::vec3 float3()
    {
        auto v = array<float>(3);
        return A::vec3(v[0], v[1], v[2]);
    }
};

struct Mesh
{
    std::vector<float> pos, nrm, uv;
    std::vector<uint32_t> idx;
};

struct Img
{
    uint32_t w = 0, h = 0;
    bool linearize = false;
    std::vector<uint8_t> px;
};

// One material property as the scene file holds it.
struct Prop
{
    std::string name;
    uint8_t kind = 0; // 1 float, 2 bool, 3 float3, 4 string, 5 float2
    float f[3]   = { 0, 0, 0 };
    bool b       = false;
    std::string s;
};

struct Material
{
    bool materialX = false;
    std::string document;
    std::vector<Prop> props;
};

int indexAfter(const std::string& s, const std::string& prefix)
{
    if (s.compare(0, prefix.size(), prefix) != 0)
        throw std::runtime_error("unexpected resource path " + s);
    return std::stoi(s.substr(prefix.size()));
}

} // namespace

int main(int argc, char** argv)
{
    bool pointers = false, lateMaterials = false, loader = false;
    for (int a = 3; a < argc; a++)
    {
        std::string opt = argv[a];
        if (opt == "--pointers")
            pointers = true;
        else if (opt == "--late-materials")
            lateMaterials = true;
        else if (opt == "--loader")
            loader = true;
        else
            argc = 0;
    }
    if (argc < 3)
    {
        std::fprintf(stderr, "usage: %s scene output [--pointers] [--late-materials] [--loader]\n", argv[0]);
        return 2;
    }
    try
    {
        Reader r;
        {
            FILE* f = std::fopen(argv[1], "rb");
            if (!f)
                throw std::runtime_error("cannot open scene file");
            std::fseek(f, 0, SEEK_END);
            r.buf.resize(size_t(std::ftell(f)));
            std::fseek(f, 0, SEEK_SET);
            if (std::fread(r.buf.data(), 1, r.buf.size(), f) != r.buf.size())
                throw std::runtime_error("cannot read scene file");
            std::fclose(f);
        }
        if (r.array<char>(4) != std::vector<char>{ 'A', 'G', 'B', 'S' })
            throw std::runtime_error("not a scene file");
        const uint32_t version = r.get<uint32_t>();
        if (version != 1 && version != 2)
            throw std::runtime_error("not a version 1 or 2 scene file");
        uint32_t width = r.get<uint32_t>(), height = r.get<uint32_t>(), spp = r.get<uint32_t>();
        uint32_t depth = r.get<uint32_t>();
        A::mat4 view = r.matrix(), proj = r.matrix();

        A::IRendererPtr renderer = A::createRenderer(A::IRenderer::Backend::Default);
        if (!renderer)
            throw std::runtime_error("createRenderer returned no renderer");
        if (renderer->backend() != A::IRenderer::Backend::Default)
            throw std::runtime_error("unexpected backend");
        A::IScenePtr scene = renderer->createScene();
        size_t loads       = 0;
        if (loader)
            renderer->setLoadResourceFunction(
                [&loads](const std::string& uri, std::vector<unsigned char>* out, std::string* name) {
                    FILE* f = std::fopen(uri.c_str(), "rb");
                    if (!f)
                        return false;
                    std::fseek(f, 0, SEEK_END);
                    out->resize(size_t(std::ftell(f)));
                    std::fseek(f, 0, SEEK_SET);
                    bool ok = std::fread(out->data(), 1, out->size(), f) == out->size();
                    std::fclose(f);
                    *name = uri;
                    loads++;
                    return ok;
                });

        // Geometry.
        std::vector<Mesh> meshes(r.get<uint32_t>());
        std::vector<A::IGeometryPtr> geometry(meshes.size());
        size_t released = 0;
        for (size_t m = 0; m < meshes.size(); m++)
        {
            Mesh& me    = meshes[m];
            uint32_t nv = r.get<uint32_t>(), ni = r.get<uint32_t>();
            me.pos      = r.array<float>(3 * size_t(nv));
            if (r.get<uint8_t>())
                me.nrm = r.array<float>(3 * size_t(nv));
            if (r.get<uint8_t>())
                me.uv = r.array<float>(2 * size_t(nv));
            me.idx = r.array<uint32_t>(ni);
            A::GeometryDescriptor d;
            d.type             = A::PrimitiveType::Triangles;
            d.vertexDesc.count = nv;
            d.vertexDesc.attributes[N::VertexAttributes::kPosition] = A::AttributeFormat::Float3;
            if (!me.nrm.empty())
                d.vertexDesc.attributes[N::VertexAttributes::kNormal] = A::AttributeFormat::Float3;
            if (!me.uv.empty())
                d.vertexDesc.attributes[N::VertexAttributes::kTexCoord0] = A::AttributeFormat::Float2;
            d.indexCount       = ni;
            // AttributeData: address, offset, size, stride.
            d.getAttributeData = [&me](A::AttributeDataMap& b, size_t, size_t, size_t, size_t) {
                b[N::VertexAttributes::kPosition] = A::AttributeData{ me.pos.data(), 0, me.pos.size() * 4, 12 };
                if (!me.nrm.empty())
                    b[N::VertexAttributes::kNormal] = A::AttributeData{ me.nrm.data(), 0, me.nrm.size() * 4, 12 };
                if (!me.uv.empty())
                    b[N::VertexAttributes::kTexCoord0] = A::AttributeData{ me.uv.data(), 0, me.uv.size() * 4, 8 };
                b[N::VertexAttributes::kIndices] = A::AttributeData{ me.idx.data(), 0, me.idx.size() * 4, 4 };
                return true;
            };
            d.attributeUpdateComplete = [&released](const A::AttributeDataMap&, size_t, size_t, size_t, size_t) {
                released++;
            };
            if (pointers)
                geometry[m] = renderer->createGeometryPointer(d, "mesh" + std::to_string(m));
            else
                scene->setGeometryDescriptor("/mesh/" + std::to_string(m), d);
        }

        // RGBA8 material textures.
        std::vector<Img> imgs(version >= 2 ? r.get<uint32_t>() : 0);
        std::vector<A::IImagePtr> images(imgs.size());
        for (size_t k = 0; k < imgs.size(); k++)
        {
            Img& im       = imgs[k];
            im.w          = r.get<uint32_t>();
            im.h          = r.get<uint32_t>();
            im.linearize  = r.get<uint8_t>() != 0;
            im.px         = r.array<uint8_t>(size_t(im.w) * im.h * 4);
            if (pointers)
            {
                A::IImage::InitData init;
                init.pImageData = im.px.data();
                init.format     = A::ImageFormat::Integer_RGBA;
                init.linearize  = im.linearize;
                init.width      = im.w;
                init.height     = im.h;
                init.name       = "image" + std::to_string(k);
                images[k]       = renderer->createImagePointer(init);
                if (!images[k])
                    throw std::runtime_error("createImagePointer failed");
                continue;
            }
            A::ImageDescriptor id;
            id.linearize = im.linearize;
            id.getData   = [&im](A::ImageData& d, A::AllocateBufferFunction) {
                d.pPixelBuffer = im.px.data();
                d.bytesPerRow  = size_t(im.w) * 4;
                d.bufferSize   = im.px.size();
                d.dimensions   = glm::ivec2(int(im.w), int(im.h));
                d.format       = A::ImageFormat::Integer_RGBA;
                return true;
            };
            scene->setImageDescriptor("/image/" + std::to_string(k), id);
        }
        // A material sampler: bilinear, wrap (the default sampler is nearest).
        A::ISamplerPtr linearSampler;
        if (version >= 2)
        {
            if (pointers)
                linearSampler = renderer->createSamplerPointer({});
            else
                scene->setSamplerProperties("/sampler/linear", {});
        }

        // Materials.
        std::vector<Material> materials(r.get<uint32_t>());
        for (Material& mat : materials)
        {
            uint32_t np = r.get<uint32_t>();
            if (np == 0xFFFFFFFFu)
            {
                auto doc      = r.array<char>(r.get<uint32_t>());
                mat.materialX = true;
                mat.document.assign(doc.begin(), doc.end());
                continue;
            }
            mat.props.resize(np);
            for (Prop& p : mat.props)
            {
                auto nameChars = r.array<char>(r.get<uint8_t>());
                p.name.assign(nameChars.begin(), nameChars.end());
                p.kind = r.get<uint8_t>();
                if (p.kind == 1)
                    p.f[0] = r.get<float>();
                else if (p.kind == 3)
                {
                    auto v = r.array<float>(3);
                    std::memcpy(p.f, v.data(), 12);
                }
                else if (p.kind == 5)
                {
                    auto v = r.array<float>(2);
                    std::memcpy(p.f, v.data(), 8);
                }
                else if (p.kind == 4)
                {
                    auto chars = r.array<char>(r.get<uint8_t>());
                    p.s.assign(chars.begin(), chars.end());
                }
                else
                    p.b = r.get<uint8_t>() != 0;
            }
        }
        std::vector<A::IMaterialPtr> matPtr(materials.size());
        if (pointers)
            for (size_t m = 0; m < materials.size(); m++)
            {
                matPtr[m] = materials[m].materialX
                    ? renderer->createMaterialPointer(N::MaterialTypes::kMaterialX, materials[m].document)
                    : renderer->createMaterialPointer();
                if (!matPtr[m])
                    throw std::runtime_error("createMaterialPointer failed");
            }
        // Sets every material's values (path-keyed: its type and properties).
        auto setMaterials = [&]() {
            for (size_t m = 0; m < materials.size(); m++)
            {
                const Material& mat = materials[m];
                if (pointers)
                {
                    A::IValues& v = matPtr[m]->values();
                    for (const Prop& p : mat.props)
                    {
                        if (p.kind == 1)
                            v.setFloat(p.name, p.f[0]);
                        else if (p.kind == 3)
                            v.setFloat3(p.name, p.f);
                        else if (p.kind == 5)
                            v.setFloat2(p.name, p.f);
                        else if (p.kind == 2)
                            v.setBoolean(p.name, p.b);
                        else if (p.s.rfind("/sampler/", 0) == 0)
                            v.setSampler(p.name, linearSampler);
                        else
                            v.setImage(p.name, images.at(size_t(indexAfter(p.s, "/image/"))));
                    }
                    continue;
                }
                A::Path path = "/material/" + std::to_string(m);
                if (mat.materialX)
                {
                    scene->setMaterialType(path, N::MaterialTypes::kMaterialX, mat.document);
                    continue;
                }
                A::Properties props;
                for (const Prop& p : mat.props)
                {
                    if (p.kind == 1)
                        props[p.name] = p.f[0];
                    else if (p.kind == 3)
                        props[p.name] = A::vec3(p.f[0], p.f[1], p.f[2]);
                    else if (p.kind == 5)
                        props[p.name] = A::vec2(p.f[0], p.f[1]);
                    else if (p.kind == 2)
                        props[p.name] = p.b;
                    else
                        props[p.name] = p.s;
                }
                scene->setMaterialType(path);
                scene->setMaterialProperties(path, props);
            }
        };
        if (!lateMaterials)
            setMaterials();

        // Instances.
        uint32_t ninst = r.get<uint32_t>();
        for (uint32_t i = 0; i < ninst; i++)
        {
            uint32_t mesh = r.get<uint32_t>(), mat = r.get<uint32_t>();
            A::mat4 xf      = r.matrix();
            A::Path path    = "/instance/" + std::to_string(i);
            std::vector<std::pair<uint32_t, uint32_t>> layers;
            if (version >= 2)
            {
                uint32_t nlayer = r.get<uint32_t>();
                for (uint32_t k = 0; k < nlayer; k++)
                {
                    uint32_t lm = r.get<uint32_t>();
                    layers.push_back({ lm, r.get<uint32_t>() });
                }
            }
            if (pointers)
            {
                A::LayerDefinitions defs;
                for (auto& l : layers)
                    defs.push_back({ matPtr.at(l.first), geometry.at(l.second) });
                if (!scene->addInstancePointer(path, geometry.at(mesh), matPtr.at(mat), xf, defs))
                    throw std::runtime_error("addInstancePointer failed");
                continue;
            }
            A::Properties ip = { { N::InstanceProperties::kMaterial, "/material/" + std::to_string(mat) },
                { N::InstanceProperties::kTransform, xf } };
            if (!layers.empty())
            {
                A::Strings lm, lg;
                for (auto& l : layers)
                {
                    lm.push_back("/material/" + std::to_string(l.first));
                    lg.push_back("/mesh/" + std::to_string(l.second));
                }
                ip[N::InstanceProperties::kMaterialLayers] = lm;
                ip[N::InstanceProperties::kGeometryLayers] = lg;
            }
            if (!scene->addInstance(path, "/mesh/" + std::to_string(mesh), ip))
                throw std::runtime_error("addInstance failed");
        }

        // Distant lights.
        uint32_t nl = r.get<uint32_t>();
        for (uint32_t l = 0; l < nl; l++)
        {
            auto v            = r.array<float>(8);
            A::ILightPtr light = scene->addLightPointer(N::LightTypes::kDistantLight);
            light->values().setFloat3(N::LightProperties::kDirection, &v[0]);
            light->values().setFloat3(N::LightProperties::kColor, &v[3]);
            light->values().setFloat(N::LightProperties::kIntensity, v[6]);
            light->values().setFloat(N::LightProperties::kAngularDiameter, v[7]);
        }

        // Environment (always path-keyed: IScene selects an environment by path).
        A::Properties envProps;
        envProps[N::EnvironmentProperties::kLightTop]         = r.float3();
        envProps[N::EnvironmentProperties::kLightBottom]      = r.float3();
        envProps[N::EnvironmentProperties::kBackgroundTop]    = r.float3();
        envProps[N::EnvironmentProperties::kBackgroundBottom] = r.float3();
        std::vector<float> envImage;
        uint32_t ew = 0, eh = 0;
        if (r.get<uint8_t>())
        {
            ew       = r.get<uint32_t>();
            eh       = r.get<uint32_t>();
            envImage = r.array<float>(3 * size_t(ew) * eh);
            A::ImageDescriptor id;
            id.isEnvironment = true;
            id.linearize     = false;
            id.getData       = [&](A::ImageData& d, A::AllocateBufferFunction) {
                d.pPixelBuffer = envImage.data();
                d.bytesPerRow  = size_t(ew) * 12;
                d.bufferSize   = envImage.size() * 4;
                d.dimensions   = glm::ivec2(int(ew), int(eh));
                d.format       = A::ImageFormat::Float_RGB;
                return true;
            };
            scene->setImageDescriptor("/environment/image", id);
            envProps[N::EnvironmentProperties::kLightImage]      = "/environment/image";
            envProps[N::EnvironmentProperties::kBackgroundImage] = "/environment/image";
        }
        if (!scene->setEnvironmentProperties("/environment", envProps) || !scene->setEnvironment("/environment"))
            throw std::runtime_error("environment rejected");
        if (r.pos < r.buf.size() && r.get<uint8_t>())
        {
            A::IGroundPlanePtr ground = renderer->createGroundPlanePointer();
            A::IValues& gv            = ground->values();
            gv.setBoolean("enabled", r.get<int32_t>() != 0);
            A::vec3 v = r.float3();
            gv.setFloat3("position", glm::value_ptr(v));
            v = r.float3();
            gv.setFloat3("normal", glm::value_ptr(v));
            gv.setFloat("shadow_opacity", r.get<float>());
            v = r.float3();
            gv.setFloat3("shadow_color", glm::value_ptr(v));
            gv.setFloat("reflection_opacity", r.get<float>());
            v = r.float3();
            gv.setFloat3("reflection_color", glm::value_ptr(v));
            gv.setFloat("reflection_roughness", r.get<float>());
            scene->setGroundPlanePointer(ground);
        }

        renderer->setScene(scene);
        renderer->setOptions({ { "traceDepth", int(depth) } });
        A::IRenderBufferPtr target = renderer->createRenderBuffer(int(width), int(height), A::ImageFormat::Float_RGBA);
        if (!target)
            throw std::runtime_error("createRenderBuffer failed");
        renderer->setTargets({ { A::AOV::kFinal, target } });
        renderer->setCamera(view, proj);
        if (lateMaterials)
        {
            renderer->render(0, 1);
            renderer->waitForTask();
            setMaterials();
        }
        renderer->render(0, spp);
        renderer->waitForTask();
        if (lateMaterials ? released < meshes.size() : released != meshes.size())
            throw std::runtime_error("attributeUpdateComplete was not called for every mesh");
        if (loader && loads == 0)
            throw std::runtime_error("the resource loader was not called");
        size_t stride   = 0;
        const float* px = static_cast<const float*>(target->data(stride));
        size_t readStride = 0;
        A::IRenderBuffer::IBufferPtr readable = target->asReadable(readStride);
        if (!readable || readStride != stride || std::memcmp(readable->data(), px, stride * height) != 0)
            throw std::runtime_error("asReadable differs from data()");
        if (stride != size_t(width) * 16)
            throw std::runtime_error("unexpected row stride");
        FILE* o = std::fopen(argv[2], "wb");
        if (!o)
            throw std::runtime_error("cannot write output");
        std::fwrite(&width, 4, 1, o);
        std::fwrite(&height, 4, 1, o);
        std::fwrite(px, 16, size_t(width) * height, o);
        std::fclose(o);
    }
    catch (const std::exception& e)
    {
        std::fprintf(stderr, "aurora_dropin_render: %s\n", e.what());
        return 1;
    }
    return 0;
}
