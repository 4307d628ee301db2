// agb_render: headless renderer over the Aurora-style C++ interface, after the Plasma
// application's batch mode (Applications/Plasma/Plasma.cpp:421-465 options, :778-790 render once
// and save): load a Wavefront OBJ or glTF 2.0 (.gltf / .glb) scene, frame the camera (or take
// --eye / --target, or --camera N for the file's N-th camera as Plasma's camera switch applies
// it, Plasma.cpp:1902-1935: its view, its vertical field of view, aspect ratio and depth range;
// orthographic cameras as glm::ortho(-xmag, xmag, -ymag, ymag, znear, zfar)), add the
// distant light and an optional lat-long Radiance HDR environment, render --output_spp samples and
// write the image (.png: the 8-bit post-processed buffer; .pfm: the float post-processed buffer).
// --ground_shadow / --ground_reflection switch on Plasma's ground plane at the scene's lower bound
// (Plasma.cpp:941-942, 989-996): matte shadow opacity 1, matte reflection opacity 0.5.
//
// usage: agb_render <scene.obj|.gltf|.glb> --output <file.png|file.pfm> [--output_spp N] [--dims W,H]
//          [--eye x,y,z] [--target x,y,z] [--up x,y,z] [--fov degrees] [--env file.hdr]
//          [--lightDir x,y,z] [--lightColor r,g,b] [--lightIntensity v] [--trace-depth N]
//          [--russian_roulette 0|1] [--gamma_correction 0|1] [--ground_shadow 0|1]
//          [--ground_reflection 0|1] [--camera N] [--mtlx file.mtlx] [--loadMtlXForObj 1]
// --mtlx applies a MaterialX document to every instance (Plasma::applyMaterialXFile,
// Plasma.cpp:1674-1703); --loadMtlXForObj takes <material>.mtlx beside an OBJ file for its OBJ
// materials (Plasma.cpp:600-605).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "aurora_gb300_loaders.hpp"

using namespace agb_aurora;

namespace
{

std::vector<float> floats(const std::string& s)
{
    std::vector<float> v;
    std::stringstream ss(s);
    std::string item;
    while (std::getline(ss, item, ','))
        v.push_back(std::strtof(item.c_str(), nullptr));
    return v;
}

vec3 vec3Arg(const std::map<std::string, std::string>& a, const std::string& key, vec3 fallback)
{
    auto it = a.find(key);
    if (it == a.end())
        return fallback;
    std::vector<float> v = floats(it->second);
    if (v.size() != 3)
        throw Error("--" + key + " takes three comma-separated numbers");
    return { v[0], v[1], v[2] };
}

vec3 sub(const vec3& a, const vec3& b) { return { a[0] - b[0], a[1] - b[1], a[2] - b[2] }; }
vec3 cross(const vec3& a, const vec3& b)
{
    return { a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0] };
}
float dot(const vec3& a, const vec3& b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
vec3 unit(const vec3& a)
{
    float l = std::sqrt(dot(a, a));
    return { a[0] / l, a[1] / l, a[2] / l };
}

// glm::lookAt and glm::perspective (right-handed, depth -1..1), column-major.
mat4 lookAt(const vec3& eye, const vec3& target, const vec3& up)
{
    vec3 f = unit(sub(target, eye));
    vec3 s = unit(cross(f, up));
    vec3 u = cross(s, f);
    return { s[0], u[0], -f[0], 0.f, s[1], u[1], -f[1], 0.f, s[2], u[2], -f[2], 0.f, -dot(s, eye),
        -dot(u, eye), dot(f, eye), 1.f };
}
mat4 perspective(float fovY, float aspect, float zNear, float zFar)
{
    float t = std::tan(fovY / 2.f);
    mat4 m{};
    m[0]  = 1.f / (aspect * t);
    m[5]  = 1.f / t;
    m[10] = -(zFar + zNear) / (zFar - zNear);
    m[11] = -1.f;
    m[14] = -(2.f * zFar * zNear) / (zFar - zNear);
    return m;
}

bool endsWith(const std::string& s, const std::string& e)
{
    return s.size() >= e.size() && s.compare(s.size() - e.size(), e.size(), e) == 0;
}

} // namespace

int main(int argc, char** argv)
{
    std::string scenePath;
    std::map<std::string, std::string> a;
    for (int i = 1; i < argc; i++)
    {
        std::string s = argv[i];
        if (s.rfind("--", 0) == 0)
        {
            if (i + 1 >= argc)
            {
                std::fprintf(stderr, "agb_render: %s needs a value\n", s.c_str());
                return 2;
            }
            a[s.substr(2)] = argv[++i];
        }
        else if (scenePath.empty())
            scenePath = s;
        else
        {
            std::fprintf(stderr, "agb_render: unexpected argument %s\n", s.c_str());
            return 2;
        }
    }
    if (scenePath.empty() || !a.count("output"))
    {
        std::fprintf(stderr,
            "usage: agb_render <scene.obj|.gltf|.glb> --output <file.png|file.pfm> [--output_spp N] [--dims W,H]\n"
            "       [--eye x,y,z] [--target x,y,z] [--up x,y,z] [--fov degrees] [--env file.hdr]\n"
            "       [--lightDir x,y,z] [--lightColor r,g,b] [--lightIntensity v] [--trace-depth N]\n"
            "       [--russian_roulette 0|1] [--gamma_correction 0|1] [--ground_shadow 0|1]\n"
            "       [--ground_reflection 0|1] [--camera N] [--mtlx file.mtlx] [--loadMtlXForObj 1]\n");
        return 2;
    }
    try
    {
        // Plasma's defaults (Plasma.h:177-228, Camera.h:75).
        int width = 1280, height = 720;
        if (a.count("dims"))
        {
            std::vector<float> d = floats(a["dims"]);
            if (d.size() != 2 || d[0] < 1 || d[1] < 1)
                throw Error("--dims takes W,H");
            width  = int(d[0]);
            height = int(d[1]);
        }
        const int spp      = a.count("output_spp") ? std::atoi(a["output_spp"].c_str()) : 64;
        const float fovY   = (a.count("fov") ? std::strtof(a["fov"].c_str(), nullptr) : 45.f) * 3.14159265f / 180.f;
        const float aspect = float(width) / float(height);

        IRendererPtr renderer = createRenderer(IRenderer::Backend::Default);
        if (!renderer)
            throw Error("no GB300 renderer available");
        IScenePtr scene = renderer->createScene();
        SceneContents contents;
        if (a.count("loadMtlXForObj"))
            loadMaterialXForOBJMaterials(std::atoi(a["loadMtlXForObj"].c_str()) != 0);
        const bool gltf = endsWith(scenePath, ".gltf") || endsWith(scenePath, ".glb");
        if (!(gltf ? loadglTFFile(scene.get(), scenePath, contents) : loadOBJFile(scene.get(), scenePath, contents)))
            throw Error("cannot load " + scenePath + (contents.warnings.empty() ? "" : ": " + contents.warnings));
        if (!contents.warnings.empty())
            std::fprintf(stderr, "%s", contents.warnings.c_str());
        if (a.count("mtlx"))
        {
            const Path material = "PlasmaMaterialX:" + a["mtlx"];
            scene->setMaterialType(material, Names::MaterialTypes::kMaterialXPath, a["mtlx"]);
            for (const SceneInstanceData& inst : contents.instances)
                scene->setInstanceProperties(inst.instance, { { Names::InstanceProperties::kMaterial, material } });
        }

        vec3 eye, target;
        fitCamera(contents.boundsMin, contents.boundsMax, { 0.f, 0.f, -1.f }, fovY, aspect, eye, target);
        eye         = vec3Arg(a, "eye", eye);
        target      = vec3Arg(a, "target", target);
        const vec3 up = vec3Arg(a, "up", { 0.f, 1.f, 0.f });

        ILightPtr light = scene->addLightPointer(Names::LightTypes::kDistantLight);
        light->values().setFloat3(Names::LightProperties::kDirection,
            unit(vec3Arg(a, "lightDir", { 1.f, -0.5f, 0.f })));
        light->values().setFloat3(Names::LightProperties::kColor, vec3Arg(a, "lightColor", { 1.f, 1.f, 1.f }));
        light->values().setFloat(Names::LightProperties::kIntensity,
            a.count("lightIntensity") ? std::strtof(a["lightIntensity"].c_str(), nullptr) : 2.f);

        std::vector<float> envPixels;
        if (a.count("env"))
        {
            int ew = 0, eh = 0;
            std::string err;
            if (!loadHDRFile(a["env"], envPixels, ew, eh, err))
                throw Error(err);
            ImageDescriptor id;
            id.getData = [&envPixels, ew, eh](ImageData& d) {
                d.pPixelBuffer = envPixels.data();
                d.bytesPerRow  = size_t(ew) * 12;
                d.bufferSize   = envPixels.size() * 4;
                d.dimensions   = { ew, eh };
                d.format       = ImageFormat::Float_RGB;
                return true;
            };
            scene->setImageDescriptor("/environment/image", id);
            scene->setEnvironmentProperties("/environment",
                { { Names::EnvironmentProperties::kLightImage, std::string("/environment/image") },
                    { Names::EnvironmentProperties::kBackgroundImage, std::string("/environment/image") } });
            scene->setEnvironment("/environment");
        }

        const bool groundShadow     = a.count("ground_shadow") && std::atoi(a["ground_shadow"].c_str()) != 0;
        const bool groundReflection = a.count("ground_reflection") && std::atoi(a["ground_reflection"].c_str()) != 0;
        if (groundShadow || groundReflection)
        {
            IGroundPlanePtr ground = renderer->createGroundPlanePointer();
            ground->values().setFloat3("position", contents.boundsMin);
            ground->values().setBoolean("enabled", true);
            ground->values().setFloat("shadow_opacity", groundShadow ? 1.f : 0.f);
            ground->values().setFloat("reflection_opacity", groundReflection ? 0.5f : 0.f);
            scene->setGroundPlanePointer(ground);
        }

        renderer->setScene(scene);
        Properties options;
        if (a.count("trace-depth"))
            options["traceDepth"] = std::atoi(a["trace-depth"].c_str());
        if (a.count("russian_roulette"))
            options["isRussianRouletteEnabled"] = std::atoi(a["russian_roulette"].c_str()) != 0;
        if (a.count("gamma_correction"))
            options["isGammaCorrectionEnabled"] = std::atoi(a["gamma_correction"].c_str()) != 0;
        renderer->setOptions(options);
        const std::string out = a["output"];
        const bool pfm        = endsWith(out, ".pfm");
        if (!pfm && !endsWith(out, ".png"))
            throw Error("--output must end in .png or .pfm");
        IRenderBufferPtr target_ =
            renderer->createRenderBuffer(width, height, pfm ? ImageFormat::Float_RGBA : ImageFormat::Integer_RGBA);
        renderer->setTargets({ { AOV::Final, target_ } });
        mat4 view = lookAt(eye, target, up), proj = perspective(fovY, aspect, 0.1f, 1000.f);
        if (a.count("camera"))
        {
            int k = std::atoi(a["camera"].c_str());
            if (k < 1 || size_t(k) > contents.cameras.size())
                throw Error("--camera " + a["camera"] + ": the scene has " + std::to_string(contents.cameras.size()) +
                    " camera(s)");
            const SceneCamera& c = contents.cameras[size_t(k - 1)];
            view                 = c.viewMatrix;
            float zn = c.znear > 0.f ? c.znear : 0.1f, zf = c.zfar > zn ? c.zfar : 1000.f;
            if (c.type == SceneCamera::Perspective)
                proj = perspective(c.yfov > 0.f ? c.yfov : fovY, c.aspectRatio > 0.f ? c.aspectRatio : aspect, zn, zf);
            else
            {
                if (!(c.xmag > 0.f && c.ymag > 0.f))
                    throw Error("--camera " + a["camera"] + ": orthographic camera without a magnification");
                proj     = mat4{};
                proj[0]  = 1.f / c.xmag;
                proj[5]  = 1.f / c.ymag;
                proj[10] = -2.f / (zf - zn);
                proj[14] = -(zf + zn) / (zf - zn);
                proj[15] = 1.f;
            }
        }
        renderer->setCamera(view, proj);
        renderer->render(0, uint32_t(spp));
        renderer->waitForTask();
        size_t stride   = 0;
        const void* px  = target_->data(stride);
        bool ok = pfm ? savePFM(out, static_cast<const float*>(px), width, height, stride)
                      : savePNG(out, static_cast<const uint8_t*>(px), width, height, stride);
        if (!ok)
            throw Error("cannot write " + out);
        std::fprintf(stderr, "agb_render: %u triangles, %d x %d, %d spp -> %s\n", contents.triangleCount, width,
            height, spp, out.c_str());
        // The camera used (column-major), exactly: lets a caller reproduce the frame.
        std::fprintf(stderr, "agb_render: view");
        for (float v : view)
            std::fprintf(stderr, " %.9g", v);
        std::fprintf(stderr, "\nagb_render: proj");
        for (float v : proj)
            std::fprintf(stderr, " %.9g", v);
        std::fprintf(stderr, "\n");
    }
    catch (const std::exception& e)
    {
        std::fprintf(stderr, "agb_render: %s\n", e.what());
        return 1;
    }
    return 0;
}
