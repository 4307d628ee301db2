// Renders a scene through the Aurora-style C++ interface (include/aurora_gb300.hpp), the way an
// Aurora client does: geometry through GeometryDescriptor callbacks, Standard Surface materials
// and instances through property maps, distant lights through ILight values, the environment
// through its properties, the camera through setCamera, then render() into an RGBA32F target.
//
// usage: aurora_api_render <scene file> <output file> [--late-materials]
// --late-materials: the scene is first rendered (1 sample) with its materials unset, then the
//   materials (and the images they name, MaterialX file images included) are set and the frame is
//   rendered again from sample 0: resources added to a scene after its first activation.
// Scene file (little-endian), written by tests/test_aurora_api.py:
//   "AGBS", u32 version (1 or 2), u32 width, height, spp, trace depth, f32 view[16], proj[16]
//     (column-major)
//   u32 meshes; per mesh: u32 vertices, indices, f32 positions[3v], u8 has normals + f32[3v],
//     u8 has uvs + f32[2v], u32 indices[i]
//   version 2: u32 images; per image: u32 width, height, u8 linearize, u8 rgba[4 * w * h]
//   u32 materials; per material: u32 properties; per property: u8 name length, name, u8 kind
//     (1 float, 3 float3, 2 bool, 4 string: u8 length + chars, 5 float2), values; or
//     u32 0xFFFFFFFF, u32 length, a MaterialX document
//   u32 instances; per instance: u32 mesh, u32 material, f32 transform[16] (column-major);
//     version 2: u32 layers; per layer: u32 material, u32 mesh with the layer's texcoords
//   u32 lights; per light: f32 direction[3], color[3], intensity, angular diameter
//   f32 light top[3], light bottom[3], background top[3], background bottom[3]
//   u8 has environment image; if set: u32 width, height, f32 rgb[3 * width * height]
//   optional: u8 has ground plane; if set: i32 enabled, f32 position[3], normal[3], shadow
//     opacity, shadow colour[3], reflection opacity, reflection colour[3], reflection roughness
// Output: u32 width, height, then f32 RGBA rows top to bottom.
#include <cstdio>
#include <cstring>
#include <functional>
#include <string>
#include <vector>

#include "aurora_gb300.hpp"

using namespace agb_aurora;

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
            throw Error("scene file truncated");
        std::memcpy(&v, &buf[pos], sizeof(T));
        pos += sizeof(T);
        return v;
    }
    template <class T>
    std::vector<T> array(size_t n)
    {
        std::vector<T> v(n);
        if (pos + n * sizeof(T) > buf.size())
            throw Error("scene file truncated");
        std::memcpy(v.data(), &buf[pos], n * sizeof(T));
        pos += n * sizeof(T);
        return v;
    }
};

struct Mesh
{
    std::vector<float> pos, nrm, uv;
    std::vector<uint32_t> idx;
};

} // namespace

int main(int argc, char** argv)
{
    if (argc != 3 && !(argc == 4 && std::string(argv[3]) == "--late-materials"))
    {
        std::fprintf(stderr, "usage: %s scene output [--late-materials]\n", argv[0]);
        return 2;
    }
    const bool lateMaterials = argc == 4;
    try
    {
        Reader r;
        {
            FILE* f = std::fopen(argv[1], "rb");
            if (!f)
                throw Error("cannot open scene file");
            std::fseek(f, 0, SEEK_END);
            r.buf.resize(size_t(std::ftell(f)));
            std::fseek(f, 0, SEEK_SET);
            if (std::fread(r.buf.data(), 1, r.buf.size(), f) != r.buf.size())
                throw Error("cannot read scene file");
            std::fclose(f);
        }
        if (r.array<char>(4) != std::vector<char>{ 'A', 'G', 'B', 'S' })
            throw Error("not a scene file");
        const uint32_t version = r.get<uint32_t>();
        if (version != 1 && version != 2)
            throw Error("not a version 1 or 2 scene file");
        uint32_t width = r.get<uint32_t>(), height = r.get<uint32_t>(), spp = r.get<uint32_t>();
        uint32_t depth = r.get<uint32_t>();
        mat4 view, proj;
        auto v16 = r.array<float>(16);
        std::memcpy(view.data(), v16.data(), 64);
        v16 = r.array<float>(16);
        std::memcpy(proj.data(), v16.data(), 64);

        IRendererPtr renderer = createRenderer(IRenderer::Backend::CUDA);
        if (!renderer)
            throw Error("no renderer");
        IScenePtr scene = renderer->createScene();

        std::vector<Mesh> meshes(r.get<uint32_t>());
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
            GeometryDescriptor d;
            d.vertexDesc.count = nv;
            d.vertexDesc.attributes[Names::VertexAttributes::kPosition] = AttributeFormat::Float3;
            if (!me.nrm.empty())
                d.vertexDesc.attributes[Names::VertexAttributes::kNormal] = AttributeFormat::Float3;
            if (!me.uv.empty())
                d.vertexDesc.attributes[Names::VertexAttributes::kTexCoord0] = AttributeFormat::Float2;
            d.indexCount       = ni;
            d.getAttributeData = [&me](AttributeDataMap& b, size_t, size_t, size_t, size_t) {
                b[Names::VertexAttributes::kPosition] = AttributeData{ me.pos.data(), me.pos.size() * 4, 0, 12 };
                if (!me.nrm.empty())
                    b[Names::VertexAttributes::kNormal] = AttributeData{ me.nrm.data(), me.nrm.size() * 4, 0, 12 };
                if (!me.uv.empty())
                    b[Names::VertexAttributes::kTexCoord0] = AttributeData{ me.uv.data(), me.uv.size() * 4, 0, 8 };
                b[Names::VertexAttributes::kIndices] = AttributeData{ me.idx.data(), me.idx.size() * 4, 0, 4 };
                return true;
            };
            d.attributeUpdateComplete = [&released](const AttributeDataMap&, size_t, size_t, size_t, size_t) {
                released++;
            };
            scene->setGeometryDescriptor("/mesh/" + std::to_string(m), d);
        }
        // Version 2: RGBA8 images /image/<k> for material textures.
        struct Img
        {
            uint32_t w = 0, h = 0;
            std::vector<uint8_t> px;
        };
        std::vector<Img> imgs(version >= 2 ? r.get<uint32_t>() : 0);
        for (size_t k = 0; k < imgs.size(); k++)
        {
            Img& im       = imgs[k];
            im.w          = r.get<uint32_t>();
            im.h          = r.get<uint32_t>();
            bool linearize = r.get<uint8_t>() != 0;
            im.px         = r.array<uint8_t>(size_t(im.w) * im.h * 4);
            ImageDescriptor id;
            id.linearize = linearize;
            id.getData   = [&im](ImageData& d) {
                d.pPixelBuffer = im.px.data();
                d.bytesPerRow  = size_t(im.w) * 4;
                d.bufferSize   = im.px.size();
                d.dimensions   = { int(im.w), int(im.h) };
                d.format       = ImageFormat::Integer_RGBA;
                return true;
            };
            scene->setImageDescriptor("/image/" + std::to_string(k), id);
        }
        if (version >= 2)
            scene->setSamplerProperties("/sampler/linear", {}); // a material sampler: bilinear, wrap
        std::vector<std::function<void()>> materialOps; // applied before or after a first render
        uint32_t nm = r.get<uint32_t>();
        for (uint32_t m = 0; m < nm; m++)
        {
            Properties props;
            uint32_t np = r.get<uint32_t>();
            if (np == 0xFFFFFFFFu)
            {
                // A MaterialX document instead of a property list.
                auto doc = r.array<char>(r.get<uint32_t>());
                Path path = "/material/" + std::to_string(m);
                std::string text(doc.begin(), doc.end());
                materialOps.push_back([scene, path, text]() {
                    scene->setMaterialType(path, Names::MaterialTypes::kMaterialX, text);
                });
                continue;
            }
            for (uint32_t k = 0; k < np; k++)
            {
                auto nameChars = r.array<char>(r.get<uint8_t>());
                std::string name(nameChars.begin(), nameChars.end());
                uint8_t kind = r.get<uint8_t>();
                if (kind == 1)
                    props[name] = r.get<float>();
                else if (kind == 3)
                {
                    auto v = r.array<float>(3);
                    props[name] = vec3{ v[0], v[1], v[2] };
                }
                else if (kind == 4)
                {
                    auto chars  = r.array<char>(r.get<uint8_t>());
                    props[name] = std::string(chars.begin(), chars.end());
                }
                else if (kind == 5)
                {
                    auto v      = r.array<float>(2);
                    props[name] = vec2{ v[0], v[1] };
                }
                else
                    props[name] = r.get<uint8_t>() != 0;
            }
            Path path = "/material/" + std::to_string(m);
            materialOps.push_back([scene, path, props]() {
                scene->setMaterialType(path);
                scene->setMaterialProperties(path, props);
            });
        }
        if (!lateMaterials)
            for (auto& op : materialOps)
                op();
        uint32_t ninst = r.get<uint32_t>();
        for (uint32_t i = 0; i < ninst; i++)
        {
            uint32_t mesh = r.get<uint32_t>(), mat = r.get<uint32_t>();
            auto t = r.array<float>(16);
            mat4 tm;
            std::memcpy(tm.data(), t.data(), 64);
            Properties ip = { { Names::InstanceProperties::kMaterial, std::string("/material/" + std::to_string(mat)) },
                { Names::InstanceProperties::kTransform, tm } };
            if (version >= 2)
            {
                // Material layers: (layer material, mesh holding the layer's texture coordinates).
                Strings lm, lg;
                uint32_t nlayer = r.get<uint32_t>();
                for (uint32_t k = 0; k < nlayer; k++)
                {
                    lm.push_back("/material/" + std::to_string(r.get<uint32_t>()));
                    lg.push_back("/mesh/" + std::to_string(r.get<uint32_t>()));
                }
                if (nlayer)
                {
                    ip[Names::InstanceProperties::kMaterialLayers] = lm;
                    ip[Names::InstanceProperties::kGeometryLayers] = lg;
                }
            }
            scene->addInstance("/instance/" + std::to_string(i), "/mesh/" + std::to_string(mesh), ip);
        }
        uint32_t nl = r.get<uint32_t>();
        for (uint32_t l = 0; l < nl; l++)
        {
            auto v          = r.array<float>(8);
            ILightPtr light = scene->addLightPointer(Names::LightTypes::kDistantLight);
            light->values().setFloat3(Names::LightProperties::kDirection, { v[0], v[1], v[2] });
            light->values().setFloat3(Names::LightProperties::kColor, { v[3], v[4], v[5] });
            light->values().setFloat(Names::LightProperties::kIntensity, v[6]);
            light->values().setFloat(Names::LightProperties::kAngularDiameter, v[7]);
        }
        auto env = r.array<float>(12);
        Properties envProps = {
            { Names::EnvironmentProperties::kLightTop, vec3{ env[0], env[1], env[2] } },
            { Names::EnvironmentProperties::kLightBottom, vec3{ env[3], env[4], env[5] } },
            { Names::EnvironmentProperties::kBackgroundTop, vec3{ env[6], env[7], env[8] } },
            { Names::EnvironmentProperties::kBackgroundBottom, vec3{ env[9], env[10], env[11] } },
        };
        std::vector<float> envImage;
        uint32_t ew = 0, eh = 0;
        if (r.get<uint8_t>())
        {
            ew       = r.get<uint32_t>();
            eh       = r.get<uint32_t>();
            envImage = r.array<float>(3 * size_t(ew) * eh);
            ImageDescriptor id;
            id.getData = [&](ImageData& d) {
                d.pPixelBuffer = envImage.data();
                d.bytesPerRow  = size_t(ew) * 12;
                d.bufferSize   = envImage.size() * 4;
                d.dimensions   = { int(ew), int(eh) };
                d.format       = ImageFormat::Float_RGB;
                return true;
            };
            scene->setImageDescriptor("/environment/image", id);
            envProps[Names::EnvironmentProperties::kLightImage]      = std::string("/environment/image");
            envProps[Names::EnvironmentProperties::kBackgroundImage] = std::string("/environment/image");
        }
        scene->setEnvironmentProperties("/environment", envProps);
        scene->setEnvironment("/environment");
        if (r.pos < r.buf.size() && r.get<uint8_t>())
        {
            IGroundPlanePtr ground = renderer->createGroundPlanePointer();
            IValues& gv            = ground->values();
            gv.setBoolean("enabled", r.get<int32_t>() != 0);
            auto f3 = [&r]() {
                auto a = r.array<float>(3);
                return vec3{ a[0], a[1], a[2] };
            };
            gv.setFloat3("position", f3());
            gv.setFloat3("normal", f3());
            gv.setFloat("shadow_opacity", r.get<float>());
            gv.setFloat3("shadow_color", f3());
            gv.setFloat("reflection_opacity", r.get<float>());
            gv.setFloat3("reflection_color", f3());
            gv.setFloat("reflection_roughness", r.get<float>());
            scene->setGroundPlanePointer(ground);
        }

        renderer->setScene(scene);
        renderer->setOptions({ { "traceDepth", int(depth) } });
        IRenderBufferPtr target = renderer->createRenderBuffer(int(width), int(height), ImageFormat::Float_RGBA);
        renderer->setTargets({ { AOV::Final, target } });
        renderer->setCamera(view, proj);
        if (lateMaterials)
        {
            renderer->render(0, 1);
            renderer->waitForTask();
            for (auto& op : materialOps)
                op();
        }
        renderer->render(0, spp);
        renderer->waitForTask();
        if (lateMaterials ? released < meshes.size() : released != meshes.size())
            throw Error("attributeUpdateComplete was not called for every mesh");
        size_t stride = 0;
        const float* px = static_cast<const float*>(target->data(stride));
        // asReadable: a copy of the same pixels; asShared: no shareable GPU image here.
        size_t readStride = 0;
        IRenderBuffer::IBufferPtr readable = target->asReadable(readStride);
        if (!readable || readStride != stride || std::memcmp(readable->data(), px, stride * height) != 0)
            throw Error("asReadable differs from data()");
        if (target->asShared() || !renderer->builtInMaterials().empty())
            throw Error("unexpected shared buffer or built-in materials");
        FILE* o = std::fopen(argv[2], "wb");
        if (!o)
            throw Error("cannot write output");
        std::fwrite(&width, 4, 1, o);
        std::fwrite(&height, 4, 1, o);
        std::fwrite(px, 16, size_t(width) * height, o);
        std::fclose(o);
    }
    catch (const std::exception& e)
    {
        std::fprintf(stderr, "aurora_api_render: %s\n", e.what());
        return 1;
    }
    return 0;
}
