// Test driver for include/aurora_gb300_loaders.hpp (no GPU needed): prints JSON.
//   loader_tool obj <file.obj>                      parse + translate, no scene
//   loader_tool gltf <file.gltf|file.glb>           parse + translate, no scene
//   loader_tool objmtlx <file.obj>                  as obj, with <material>.mtlx files beside it
//   loader_tool gltfsave <out.gltf> <in.gltf>       the input's cameras written as a glTF file
//   loader_tool mtlx <file.mtlx>                    standard_surface constants as properties
//   loader_tool pngread <file.png>                  decoded 8-bit RGBA
//   loader_tool hdr <file.hdr>                      width, height, RGB floats
//   loader_tool png <out.png> <w> <h>               writes a pattern image
//   loader_tool pfm <out.pfm> <w> <h>               writes a pattern image
//   loader_tool fit <min xyz> <max xyz> <dir xyz> <fovY rad> <aspect>
#include <cstdio>
#include <cstdlib>
#include <string>
#include <variant>
#include <vector>

#include "aurora_gb300_loaders.hpp"

using namespace agb_aurora;

namespace
{

void printFloats(const float* v, size_t n)
{
    std::printf("[");
    for (size_t i = 0; i < n; i++)
        std::printf("%s%.9g", i ? "," : "", v[i]);
    std::printf("]");
}

void printString(const std::string& s)
{
    std::printf("\"");
    for (char c : s)
    {
        if (c == '"' || c == '\\')
            std::printf("\\%c", c);
        else if (c == '\n')
            std::printf("\\n");
        else
            std::printf("%c", c);
    }
    std::printf("\"");
}

void printValue(const PropertyValue& v)
{
    if (std::holds_alternative<bool>(v))
        std::printf("%s", std::get<bool>(v) ? "true" : "false");
    else if (std::holds_alternative<int>(v))
        std::printf("%d", std::get<int>(v));
    else if (std::holds_alternative<float>(v))
        std::printf("%.9g", std::get<float>(v));
    else if (std::holds_alternative<vec2>(v))
        printFloats(std::get<vec2>(v).data(), 2);
    else if (std::holds_alternative<vec3>(v))
        printFloats(std::get<vec3>(v).data(), 3);
    else if (std::holds_alternative<Strings>(v))
    {
        std::printf("[");
        const Strings& list = std::get<Strings>(v);
        for (size_t i = 0; i < list.size(); i++)
        {
            std::printf("%s", i ? "," : "");
            printString(list[i]);
        }
        std::printf("]");
    }
    else if (std::holds_alternative<mat4>(v))
        printFloats(std::get<mat4>(v).data(), 16);
    else if (std::holds_alternative<std::monostate>(v))
        std::printf("null");
    else
        printString(std::get<std::string>(v));
}

} // namespace

int main(int argc, char** argv)
{
    if (argc < 3)
        return 2;
    std::string mode = argv[1];
    if (mode == "pngread")
    {
        std::vector<uint8_t> rgba;
        int w = 0, h = 0;
        std::string err;
        bool ok = loadPNGFile(argv[2], rgba, w, h, err);
        std::printf("{\"ok\":%s,\"error\":", ok ? "true" : "false");
        printString(err);
        std::printf(",\"width\":%d,\"height\":%d,\"rgba\":[", w, h);
        for (size_t i = 0; i < rgba.size(); i++)
            std::printf("%s%u", i ? "," : "", unsigned(rgba[i]));
        std::printf("]}\n");
        return 0;
    }
    if (mode == "mtlx")
    {
        Properties props;
        std::string warnings;
        std::vector<MaterialXImage> images;
        bool ok = materialXFileToProperties(argv[2], props, warnings, &images);
        std::printf("{\"ok\":%s,\"warnings\":", ok ? "true" : "false");
        printString(warnings);
        std::printf(",\"images\":[");
        for (size_t i = 0; i < images.size(); i++)
        {
            std::printf("%s{\"property\":", i ? "," : "");
            printString(images[i].property);
            std::printf(",\"image\":");
            printString(images[i].image);
            std::printf(",\"file\":");
            printString(images[i].file);
            std::printf(",\"linearize\":%s}", images[i].linearize ? "true" : "false");
        }
        std::printf("]");
        std::printf(",\"properties\":{");
        bool first = true;
        for (auto& kv : props)
        {
            std::printf("%s", first ? "" : ",");
            first = false;
            printString(kv.first);
            std::printf(":");
            printValue(kv.second);
        }
        std::printf("}}\n");
        return 0;
    }
    if (mode == "gltfsave" && argc == 4)
    {
        // Loads the cameras of argv[3] and writes them to argv[2].
        SceneContents c;
        if (!loadglTFFile(nullptr, argv[3], c))
            return 1;
        return saveglTFFile(argv[2], c) ? 0 : 1;
    }
    if (mode == "obj" || mode == "gltf" || mode == "objmtlx")
    {
        SceneContents c;
        loadMaterialXForOBJMaterials(mode == "objmtlx");
        bool ok = mode != "gltf" ? loadOBJFile(nullptr, argv[2], c) : loadglTFFile(nullptr, argv[2], c);
        std::printf("{\"ok\":%s,\"warnings\":", ok ? "true" : "false");
        printString(c.warnings);
        std::printf(",\"bounds\":[");
        printFloats(c.boundsMin.data(), 3);
        std::printf(",");
        printFloats(c.boundsMax.data(), 3);
        std::printf("],\"materials\":[");
        for (size_t i = 0; i < c.materials.size(); i++)
        {
            std::printf("%s{\"path\":", i ? "," : "");
            printString(c.materials[i].path);
            std::printf(",\"properties\":{");
            bool first = true;
            for (auto& kv : c.materials[i].properties)
            {
                std::printf("%s", first ? "" : ",");
                first = false;
                printString(kv.first);
                std::printf(":");
                printValue(kv.second);
            }
            std::printf("}}");
        }
        std::printf("],\"instances\":[");
        for (size_t i = 0; i < c.instances.size(); i++)
        {
            const SceneGeometryData& g = c.geometry[c.instances[i].geometry];
            std::printf("%s{\"instance\":", i ? "," : "");
            printString(c.instances[i].instance);
            std::printf(",\"material\":");
            printString(c.instances[i].material);
            std::printf(",\"geometry\":");
            printString(c.instances[i].geometry);
            std::printf(",\"transform\":");
            printFloats(c.instances[i].transform.data(), 16);
            std::printf(",\"positions\":");
            printFloats(g.positions.data(), g.positions.size());
            std::printf(",\"normals\":");
            printFloats(g.normals.data(), g.normals.size());
            std::printf(",\"texcoords\":");
            printFloats(g.texCoords.data(), g.texCoords.size());
            std::printf(",\"indices\":[");
            for (size_t k = 0; k < g.indices.size(); k++)
                std::printf("%s%u", k ? "," : "", g.indices[k]);
            std::printf("]}");
        }
        std::printf("],\"images\":[");
        for (size_t i = 0; i < c.images.size(); i++)
        {
            std::printf("%s{\"path\":", i ? "," : "");
            printString(c.images[i].path);
            std::printf(",\"file\":");
            printString(c.images[i].file);
            std::printf(",\"linearize\":%s}", c.images[i].linearize ? "true" : "false");
        }
        std::printf("],\"cameras\":[");
        for (size_t i = 0; i < c.cameras.size(); i++)
        {
            const SceneCamera& k = c.cameras[i];
            std::printf("%s{\"name\":", i ? "," : "");
            printString(k.name);
            std::printf(",\"type\":\"%s\",\"view\":", k.type == SceneCamera::Perspective ? "perspective" : "orthographic");
            printFloats(k.viewMatrix.data(), 16);
            float v[6] = { k.yfov, k.aspectRatio, k.xmag, k.ymag, k.znear, k.zfar };
            std::printf(",\"values\":");
            printFloats(v, 6);
            std::printf("}");
        }
        std::printf("],\"vertices\":%u,\"triangles\":%u}\n", c.vertexCount, c.triangleCount);
        return 0;
    }
    if (mode == "hdr")
    {
        std::vector<float> rgb;
        int w = 0, h = 0;
        std::string err;
        bool ok = loadHDRFile(argv[2], rgb, w, h, err);
        std::printf("{\"ok\":%s,\"error\":", ok ? "true" : "false");
        printString(err);
        std::printf(",\"width\":%d,\"height\":%d,\"rgb\":", w, h);
        printFloats(rgb.data(), rgb.size());
        std::printf("}\n");
        return 0;
    }
    if ((mode == "png" || mode == "pfm") && argc == 5)
    {
        int w = std::atoi(argv[3]), h = std::atoi(argv[4]);
        if (mode == "png")
        {
            std::vector<uint8_t> px(size_t(w) * h * 4);
            for (size_t i = 0; i < px.size(); i++)
                px[i] = uint8_t((i * 37u + i / 7u) & 0xffu);
            return savePNG(argv[2], px.data(), w, h, size_t(w) * 4) ? 0 : 1;
        }
        std::vector<float> px(size_t(w) * h * 4);
        for (size_t i = 0; i < px.size(); i++)
            px[i] = float(i) * 0.25f - 3.f;
        return savePFM(argv[2], px.data(), w, h, size_t(w) * 16) ? 0 : 1;
    }
    if (mode == "fit" && argc == 13)
    {
        vec3 bmin = { float(std::atof(argv[2])), float(std::atof(argv[3])), float(std::atof(argv[4])) };
        vec3 bmax = { float(std::atof(argv[5])), float(std::atof(argv[6])), float(std::atof(argv[7])) };
        vec3 dir  = { float(std::atof(argv[8])), float(std::atof(argv[9])), float(std::atof(argv[10])) };
        vec3 eye, target;
        fitCamera(bmin, bmax, dir, float(std::atof(argv[11])), float(std::atof(argv[12])), eye, target);
        std::printf("{\"eye\":");
        printFloats(eye.data(), 3);
        std::printf(",\"target\":");
        printFloats(target.data(), 3);
        std::printf("}\n");
        return 0;
    }
    return 2;
}
