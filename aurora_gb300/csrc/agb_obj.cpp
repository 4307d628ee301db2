// Scene and image I/O of the headless renderer (declarations and provenance in
// include/aurora_gb300_loaders.hpp): OBJ / MTL parsing and translation, smooth normals, Radiance
// HDR reading, PNG and PFM writing, camera fit.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <unordered_map>

#include "../../include/aurora_gb300_loaders.hpp"

namespace agb_aurora
{
namespace
{

bool readWholeFile(const std::string& path, std::string& out)
{
    std::ifstream f(path, std::ios::binary);
    if (!f)
        return false;
    std::ostringstream s;
    s << f.rdbuf();
    out = s.str();
    return true;
}

std::string directoryOf(const std::string& path)
{
    size_t k = path.find_last_of("/\\");
    return k == std::string::npos ? std::string() : path.substr(0, k + 1);
}

// Splits a line into whitespace-separated tokens.
std::vector<std::string> tokens(const std::string& line)
{
    std::vector<std::string> out;
    std::istringstream s(line);
    std::string t;
    while (s >> t)
        out.push_back(t);
    return out;
}

bool toFloat(const std::string& s, float& v)
{
    char* end = nullptr;
    v         = std::strtof(s.c_str(), &end);
    return end && end != s.c_str();
}

// The remainder of a texture record after its options: the file name is the last token.
std::string textureName(const std::vector<std::string>& t)
{
    return t.size() >= 2 ? t.back() : std::string();
}

void parseMTL(const std::string& text, std::vector<ObjMaterial>& mats, std::string& warnings)
{
    std::istringstream in(text);
    std::string line;
    ObjMaterial* m = nullptr;
    while (std::getline(in, line))
    {
        if (!line.empty() && line.back() == '\r')
            line.pop_back();
        std::vector<std::string> t = tokens(line);
        if (t.empty() || t[0][0] == '#')
            continue;
        const std::string& k = t[0];
        if (k == "newmtl")
        {
            mats.emplace_back();
            m       = &mats.back();
            m->name = t.size() > 1 ? t[1] : std::string();
            continue;
        }
        if (!m)
            continue;
        auto color = [&](float* c) {
            float v;
            for (int i = 0; i < 3; i++)
                c[i] = (t.size() > size_t(1 + i) && toFloat(t[1 + i], v)) ? v : (i > 0 ? c[0] : 0.f);
        };
        float v = 0.f;
        if (k == "Kd")
            color(m->diffuse);
        else if (k == "Ks")
            color(m->specular);
        else if (k == "Tf" || k == "Kt")
            color(m->transmittance);
        else if (k == "Ke")
            color(m->emission);
        else if (k == "Ni" && t.size() > 1 && toFloat(t[1], v))
            m->ior = v;
        else if (k == "d" && t.size() > 1 && toFloat(t[1], v))
            m->dissolve = v;
        else if (k == "Tr" && t.size() > 1 && toFloat(t[1], v))
            m->dissolve = 1.f - v;
        else if (k == "Pr" && t.size() > 1 && toFloat(t[1], v))
            m->roughness = v;
        else if (k == "Pm" && t.size() > 1 && toFloat(t[1], v))
            m->metallic = v;
        else if (k == "map_Kd")
            m->diffuseTex = textureName(t);
        else if (k == "map_Pr")
            m->roughnessTex = textureName(t);
        else if (k == "map_Ke")
            m->emissiveTex = textureName(t);
        else if (k == "map_d")
            m->alphaTex = textureName(t);
        else if (k == "bump" || k == "map_bump" || k == "map_Bump")
            m->bumpTex = textureName(t);
        else if (k == "norm")
            m->normalTex = textureName(t);
    }
    (void)warnings;
}

// OBJ index field "v", "v/vt", "v//vn" or "v/vt/vn"; 1-based, negative = relative to the end.
bool parseIndex(const std::string& s, size_t nv, size_t nt, size_t nn, ObjIndex& out)
{
    int fields[3]  = { 0, 0, 0 };
    bool present[3] = { false, false, false };
    size_t pos      = 0;
    for (int f = 0; f < 3 && pos <= s.size(); f++)
    {
        size_t slash = s.find('/', pos);
        std::string part = s.substr(pos, slash == std::string::npos ? std::string::npos : slash - pos);
        if (!part.empty())
        {
            char* end = nullptr;
            long v    = std::strtol(part.c_str(), &end, 10);
            if (!end || *end != '\0' || v == 0)
                return false;
            fields[f]  = int(v);
            present[f] = true;
        }
        if (slash == std::string::npos)
            break;
        pos = slash + 1;
    }
    if (!present[0])
        return false;
    const size_t counts[3] = { nv, nt, nn };
    int* dst[3]            = { &out.position, &out.texcoord, &out.normal };
    for (int f = 0; f < 3; f++)
    {
        if (!present[f])
        {
            *dst[f] = -1;
            continue;
        }
        long idx = fields[f] > 0 ? long(fields[f]) - 1 : long(counts[f]) + fields[f];
        if (idx < 0)
            return false;
        *dst[f] = int(idx);
    }
    return true;
}

float sRGBToLinear(float v)
{
    // Plasma/pch.h:124-128 (a cubic fit).
    return v * (v * (v * 0.305306011f + 0.682171111f) + 0.012522878f);
}
vec3 sRGBToLinear3(const float* c) { return { sRGBToLinear(c[0]), sRGBToLinear(c[1]), sRGBToLinear(c[2]) }; }
float length3(const vec3& v) { return std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); }

struct IndexKey
{
    int p, n, t;
    bool operator==(const IndexKey& o) const { return p == o.p && n == o.n && t == o.t; }
};
struct IndexKeyHash
{
    size_t operator()(const IndexKey& k) const
    {
        return (size_t(uint32_t(k.p)) * 73856093u) ^ (size_t(uint32_t(k.n)) * 19349663u) ^
            (size_t(uint32_t(k.t)) * 83492791u);
    }
};

uint32_t crc32(const uint8_t* p, size_t n, uint32_t c = 0xffffffffu)
{
    for (size_t i = 0; i < n; i++)
    {
        c ^= p[i];
        for (int k = 0; k < 8; k++)
            c = (c >> 1) ^ (0xedb88320u & (0u - (c & 1u)));
    }
    return c;
}

} // namespace

bool parseOBJ(const std::string& text, const std::function<bool(const std::string&, std::string&)>& readFile,
    ObjData& out, std::string& error)
{
    out = ObjData();
    std::istringstream in(text);
    std::string line;
    int currentMaterial = -1;
    std::unordered_map<std::string, int> materialIds;
    ObjShape shape;
    auto flush = [&]() {
        if (!shape.indices.empty())
            out.shapes.push_back(shape);
        shape.indices.clear();
        shape.materialIds.clear();
    };
    size_t lineNo = 0;
    while (std::getline(in, line))
    {
        lineNo++;
        if (!line.empty() && line.back() == '\r')
            line.pop_back();
        std::vector<std::string> t = tokens(line);
        if (t.empty() || t[0][0] == '#')
            continue;
        const std::string& k = t[0];
        float v[3];
        if (k == "v" || k == "vn")
        {
            if (t.size() < 4 || !toFloat(t[1], v[0]) || !toFloat(t[2], v[1]) || !toFloat(t[3], v[2]))
            {
                error = "line " + std::to_string(lineNo) + ": bad " + k + " record";
                return false;
            }
            std::vector<float>& dst = k == "v" ? out.positions : out.normals;
            dst.insert(dst.end(), v, v + 3);
        }
        else if (k == "vt")
        {
            if (t.size() < 2 || !toFloat(t[1], v[0]))
            {
                error = "line " + std::to_string(lineNo) + ": bad vt record";
                return false;
            }
            v[1] = (t.size() > 2 && toFloat(t[2], v[1])) ? v[1] : 0.f;
            out.texcoords.push_back(v[0]);
            out.texcoords.push_back(v[1]);
        }
        else if (k == "f")
        {
            std::vector<ObjIndex> poly;
            for (size_t i = 1; i < t.size(); i++)
            {
                ObjIndex idx;
                if (!parseIndex(t[i], out.positions.size() / 3, out.texcoords.size() / 2,
                        out.normals.size() / 3, idx))
                {
                    error = "line " + std::to_string(lineNo) + ": bad face index '" + t[i] + "'";
                    return false;
                }
                poly.push_back(idx);
            }
            if (poly.size() < 3)
            {
                out.warnings += "line " + std::to_string(lineNo) + ": face with fewer than 3 vertices skipped\n";
                continue;
            }
            for (size_t i = 1; i + 1 < poly.size(); i++)
            {
                shape.indices.push_back(poly[0]);
                shape.indices.push_back(poly[i]);
                shape.indices.push_back(poly[i + 1]);
                shape.materialIds.push_back(currentMaterial);
            }
        }
        else if (k == "o" || k == "g")
        {
            flush();
            shape.name = t.size() > 1 ? line.substr(line.find(t[1])) : std::string();
        }
        else if (k == "usemtl")
        {
            auto it         = materialIds.find(t.size() > 1 ? t[1] : std::string());
            currentMaterial = it == materialIds.end() ? -1 : it->second;
            if (it == materialIds.end())
                out.warnings += "line " + std::to_string(lineNo) + ": unknown material\n";
        }
        else if (k == "mtllib")
        {
            for (size_t i = 1; i < t.size(); i++)
            {
                std::string mtl;
                if (!readFile || !readFile(t[i], mtl))
                {
                    out.warnings += "material library '" + t[i] + "' not found\n";
                    continue;
                }
                size_t before = out.materials.size();
                parseMTL(mtl, out.materials, out.warnings);
                for (size_t m = before; m < out.materials.size(); m++)
                    materialIds[out.materials[m].name] = int(m);
            }
        }
    }
    flush();
    return true;
}

void calculateNormals(size_t vertexCount, const float* positions, size_t triangleCount,
    const uint32_t* indices, float* normalsOut)
{
    auto load = [&](uint32_t i) { return vec3{ positions[3 * i], positions[3 * i + 1], positions[3 * i + 2] }; };
    auto sub  = [](const vec3& a, const vec3& b) { return vec3{ a[0] - b[0], a[1] - b[1], a[2] - b[2] }; };
    auto dot  = [](const vec3& a, const vec3& b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; };
    auto unit = [&](const vec3& a) {
        float l = std::sqrt(dot(a, a));
        return vec3{ a[0] / l, a[1] / l, a[2] / l };
    };
    std::fill(normalsOut, normalsOut + 3 * vertexCount, 0.f);
    for (size_t f = 0; f < triangleCount; f++)
    {
        uint32_t i1 = indices[3 * f], i2 = indices[3 * f + 1], i3 = indices[3 * f + 2];
        vec3 p1 = load(i1), p2 = load(i2), p3 = load(i3);
        vec3 e12 = sub(p2, p1), e13 = sub(p3, p1);
        vec3 n   = unit(vec3{ e12[1] * e13[2] - e12[2] * e13[1], e12[2] * e13[0] - e12[0] * e13[2],
              e12[0] * e13[1] - e12[1] * e13[0] });
        // Corner weights as the reference computes them: the angles between (p3 - p1, p2 - p1),
        // (p3 - p2, p2 - p1) and (p1 - p3, p2 - p3).
        vec3 u13 = unit(e13), u12 = unit(e12), u23 = unit(sub(p3, p2));
        float w[3] = { std::fabs(std::acos(dot(u13, u12))), std::fabs(std::acos(dot(u23, u12))),
            std::fabs(std::acos(dot(u13, u23))) };
        uint32_t ids[3] = { i1, i2, i3 };
        for (int c = 0; c < 3; c++)
            for (int k = 0; k < 3; k++)
                normalsOut[3 * ids[c] + k] += n[k] * w[c];
    }
    for (size_t i = 0; i < vertexCount; i++)
    {
        vec3 n = unit(vec3{ normalsOut[3 * i], normalsOut[3 * i + 1], normalsOut[3 * i + 2] });
        std::memcpy(normalsOut + 3 * i, n.data(), sizeof(float) * 3);
    }
}

namespace
{
bool gMaterialXForOBJ = false;
}

void loadMaterialXForOBJMaterials(bool enabled) { gMaterialXForOBJ = enabled; }

bool translateOBJ(const ObjData& obj, const std::string& filePath, SceneContents& contents)
{
    contents.reset();
    std::vector<Path> materialPaths;
    int mtlCount = 0;
    for (const ObjMaterial& m : obj.materials)
    {
        if (gMaterialXForOBJ && !m.name.empty())
        {
            const std::string mtlx = directoryOf(filePath) + m.name + ".mtlx";
            if (std::ifstream(mtlx).good())
            {
                SceneMaterialData md;
                md.path = filePath + "-" + m.name + ":MaterialX-" + std::to_string(mtlCount++);
                std::vector<MaterialXImage> imgs;
                if (materialXFileToProperties(mtlx, md.properties, contents.warnings, &imgs))
                {
                    for (const MaterialXImage& im : imgs)
                        contents.images.push_back(SceneImageData{ im.image, im.file, im.linearize });
                    materialPaths.push_back(md.path);
                    contents.materials.push_back(std::move(md));
                    continue;
                }
            }
        }
        // OBJLoader.cpp:155-232: Standard Surface values from the MTL record.
        vec3 baseColor         = sRGBToLinear3(m.diffuse);
        vec3 specularColor     = sRGBToLinear3(m.specular);
        float specularIOR      = m.ior == 1.0f ? 1.5f : m.ior;
        float transmission     = 1.0f - m.dissolve;
        vec3 transmissionColor = sRGBToLinear3(m.transmittance);
        if (length3(transmissionColor) == 0.0f)
            transmissionColor = { 1.f, 1.f, 1.f };
        vec3 emissionColor = sRGBToLinear3(m.emission);
        // ImageCache::getImage (Loaders.h:22-38): one image path per (file, linearize).
        auto image = [&](const std::string& name, bool linearize) -> Path {
            if (name.empty())
                return Path();
            Path p = "PlasmaImage/" + name + ":linearize:" + std::to_string(linearize ? 1 : 0);
            for (const SceneImageData& im : contents.images)
                if (im.path == p)
                    return p;
            contents.images.push_back(SceneImageData{ p, directoryOf(filePath) + name, linearize });
            return p;
        };
        Path baseColorImage         = image(m.diffuseTex, true);
        Path specularRoughnessImage = image(m.roughnessTex, false);
        Path emissionColorImage     = image(m.emissiveTex, true);
        Path opacityImage           = image(m.alphaTex, false);
        Path normalImage            = image(m.normalTex.empty() ? m.bumpTex : m.normalTex, false);
        float emission = (!emissionColorImage.empty() || length3(emissionColor) != 0.0f) ? 1.0f : 0.0f;
        SceneMaterialData md;
        md.path       = filePath + "-" + m.name + ":OBJFileMaterial-" + std::to_string(mtlCount++);
        md.properties = {
            { "base_color", baseColor },
            { "metalness", m.metallic },
            { "specular_color", specularColor },
            { "specular_roughness", m.roughness },
            { "specular_IOR", specularIOR },
            { "transmission", transmission },
            { "transmission_color", transmissionColor },
            { "emission", emission },
            { "emission_color", emissionColor },
            { "opacity", vec3{ 1.f, 1.f, 1.f } },
            { "base_color_image", baseColorImage },
            { "specular_roughness_image", specularRoughnessImage },
            { "emission_color_image", emissionColorImage },
            { "opacity_image", opacityImage },
            { "normal_image", normalImage },
        };
        materialPaths.push_back(md.path);
        contents.materials.push_back(std::move(md));
    }
    bool hasMesh  = false;
    bool first    = true;
    uint32_t objectCount = 0;
    for (const ObjShape& shape : obj.shapes)
    {
        if (shape.indices.empty())
            continue;
        hasMesh            = true;
        Path instancePath  = filePath + "-" + shape.name + ":OBJFileInstance-" + std::to_string(objectCount);
        Path geomPath      = filePath + "-" + shape.name + ":OBJFileGeom-" + std::to_string(objectCount);
        objectCount++;
        SceneGeometryData& g = contents.geometry[geomPath];
        const bool hasNormals   = shape.indices[0].normal >= 0;
        const bool hasTexCoords = shape.indices[0].texcoord >= 0;
        std::unordered_map<IndexKey, uint32_t, IndexKeyHash> unique;
        for (const ObjIndex& oi : shape.indices)
        {
            IndexKey key{ oi.position, oi.normal, oi.texcoord };
            auto it = unique.find(key);
            if (it != unique.end())
            {
                g.indices.push_back(it->second);
                continue;
            }
            // OBJLoader.cpp:300-356: skip corners whose sub-indices are out of range.
            if (size_t(oi.position) * 3 + 3 > obj.positions.size() ||
                (hasNormals && (oi.normal < 0 || size_t(oi.normal) * 3 >= obj.normals.size())) ||
                (hasTexCoords && (oi.texcoord < 0 || size_t(oi.texcoord) * 2 >= obj.texcoords.size())))
            {
                contents.warnings += "invalid index in shape '" + shape.name + "'\n";
                continue;
            }
            const float* p = &obj.positions[3 * size_t(oi.position)];
            for (int k = 0; k < 3; k++)
            {
                contents.boundsMin[k] = first ? p[k] : std::min(contents.boundsMin[k], p[k]);
                contents.boundsMax[k] = first ? p[k] : std::max(contents.boundsMax[k], p[k]);
            }
            first = false;
            g.positions.insert(g.positions.end(), p, p + 3);
            if (hasNormals)
            {
                const float* n = &obj.normals[3 * size_t(oi.normal)];
                float l        = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
                g.normals.push_back(n[0] / l);
                g.normals.push_back(n[1] / l);
                g.normals.push_back(n[2] / l);
            }
            if (hasTexCoords)
            {
                const float* uv = &obj.texcoords[2 * size_t(oi.texcoord)];
                g.texCoords.push_back(uv[0]);
                g.texCoords.push_back(1.0f - uv[1]); // flip V
            }
            uint32_t id = uint32_t(g.positions.size() / 3 - 1);
            unique.emplace(key, id);
            g.indices.push_back(id);
        }
        // A skipped corner leaves a partial triangle: keep whole triangles only.
        g.indices.resize(g.indices.size() - g.indices.size() % 3);
        uint32_t vertexCount = uint32_t(g.positions.size() / 3);
        if (!hasNormals)
        {
            g.normals.resize(g.positions.size());
            calculateNormals(vertexCount, g.positions.data(), g.indices.size() / 3, g.indices.data(),
                g.normals.data());
        }
        SceneInstanceData inst;
        inst.instance = instancePath;
        inst.geometry = geomPath;
        int mid       = shape.materialIds.empty() ? -1 : shape.materialIds[0];
        if (mid >= 0)
        {
            if (size_t(mid) >= materialPaths.size())
                mid = 0;
            inst.material = materialPaths[size_t(mid)];
        }
        contents.instances.push_back(inst);
        contents.vertexCount += vertexCount;
        contents.triangleCount += uint32_t(g.indices.size() / 3);
    }
    contents.warnings = obj.warnings + contents.warnings;
    return hasMesh;
}

bool loadOBJFile(IScene* scene, const std::string& filePath, SceneContents& contents)
{
    contents.reset();
    std::string text;
    if (!readWholeFile(filePath, text))
        return false;
    const std::string dir = directoryOf(filePath);
    ObjData obj;
    std::string error;
    if (!parseOBJ(text, [&](const std::string& name, std::string& out) { return readWholeFile(dir + name, out); },
            obj, error))
    {
        contents.warnings = error;
        return false;
    }
    if (!translateOBJ(obj, filePath, contents))
        return false;
    addContentsToScene(scene, contents);
    return true;
}

void addContentsToScene(IScene* scene, SceneContents& contents)
{
    if (!scene)
        return;
    for (const SceneImageData& im : contents.images)
        scene->setImageFromFilePath(im.path, im.file, im.linearize);
    for (const SceneMaterialData& m : contents.materials)
    {
        scene->setMaterialType(m.path);
        scene->setMaterialProperties(m.path, m.properties);
    }
    for (const SceneInstanceData& inst : contents.instances)
    {
        SceneGeometryData& g = contents.geometry[inst.geometry];
        GeometryDescriptor d;
        d.vertexDesc.count = g.positions.size() / 3;
        d.vertexDesc.attributes[Names::VertexAttributes::kPosition] = AttributeFormat::Float3;
        d.vertexDesc.attributes[Names::VertexAttributes::kNormal]   = AttributeFormat::Float3;
        if (!g.texCoords.empty())
            d.vertexDesc.attributes[Names::VertexAttributes::kTexCoord0] = AttributeFormat::Float2;
        d.indexCount       = g.indices.size();
        d.getAttributeData = [&g](AttributeDataMap& b, size_t, size_t, size_t, size_t) {
            b[Names::VertexAttributes::kPosition] = AttributeData{ g.positions.data(), g.positions.size() * 4, 0, 12 };
            b[Names::VertexAttributes::kNormal]   = AttributeData{ g.normals.data(), g.normals.size() * 4, 0, 12 };
            if (!g.texCoords.empty())
                b[Names::VertexAttributes::kTexCoord0] = AttributeData{ g.texCoords.data(), g.texCoords.size() * 4, 0, 8 };
            b[Names::VertexAttributes::kIndices] = AttributeData{ g.indices.data(), g.indices.size() * 4, 0, 4 };
            return true;
        };
        scene->setGeometryDescriptor(inst.geometry, d);
        Properties props = { { Names::InstanceProperties::kTransform, inst.transform } };
        if (!inst.material.empty())
            props[Names::InstanceProperties::kMaterial] = inst.material;
        scene->addInstance(inst.instance, inst.geometry, props);
    }
    scene->setBounds(contents.boundsMin, contents.boundsMax);
}

bool loadHDRFile(const std::string& path, std::vector<float>& rgb, int& width, int& height, std::string& error)
{
    std::string data;
    if (!readWholeFile(path, data))
    {
        error = "cannot read " + path;
        return false;
    }
    return decodeHDR(data, rgb, width, height, error);
}

bool decodeHDR(const std::string& data, std::vector<float>& rgb, int& width, int& height, std::string& error)
{
    size_t pos = 0;
    auto nextLine = [&](std::string& l) {
        size_t e = data.find('\n', pos);
        if (e == std::string::npos)
            return false;
        l   = data.substr(pos, e - pos);
        pos = e + 1;
        return true;
    };
    std::string l;
    if (!nextLine(l) || (l.rfind("#?RADIANCE", 0) != 0 && l.rfind("#?RGBE", 0) != 0))
    {
        error = "not a Radiance HDR file";
        return false;
    }
    while (nextLine(l) && !l.empty())
        if (l.rfind("FORMAT=", 0) == 0 && l != "FORMAT=32-bit_rle_rgbe")
        {
            error = "unsupported HDR format " + l;
            return false;
        }
    char ya[3] = { 0 }, xa[3] = { 0 };
    if (!nextLine(l) || std::sscanf(l.c_str(), "%2s %d %2s %d", ya, &height, xa, &width) != 4 ||
        std::string(ya) != "-Y" || std::string(xa) != "+X" || width <= 0 || height <= 0 ||
        size_t(width) * size_t(height) > (size_t(1) << 30))
    {
        error = "unsupported HDR orientation or size";
        return false;
    }
    const uint8_t* p   = reinterpret_cast<const uint8_t*>(data.data()) + pos;
    const uint8_t* end = reinterpret_cast<const uint8_t*>(data.data()) + data.size();
    rgb.assign(size_t(width) * height * 3, 0.f);
    std::vector<uint8_t> line(size_t(width) * 4);
    for (int y = 0; y < height; y++)
    {
        bool rle = width >= 8 && width < 32768 && end - p >= 4 && p[0] == 2 && p[1] == 2 && (p[2] & 0x80) == 0;
        if (rle)
        {
            if (((p[2] << 8) | p[3]) != width)
            {
                error = "bad HDR scanline";
                return false;
            }
            p += 4;
            for (int c = 0; c < 4; c++)
                for (int x = 0; x < width;)
                {
                    if (p >= end)
                    {
                        error = "truncated HDR data";
                        return false;
                    }
                    int n = *p++;
                    if (n > 128)
                    {
                        n -= 128;
                        if (p >= end || x + n > width)
                        {
                            error = "bad HDR run";
                            return false;
                        }
                        uint8_t v = *p++;
                        for (int i = 0; i < n; i++)
                            line[size_t(x++) * 4 + c] = v;
                    }
                    else
                    {
                        if (n == 0 || end - p < n || x + n > width)
                        {
                            error = "bad HDR run";
                            return false;
                        }
                        for (int i = 0; i < n; i++)
                            line[size_t(x++) * 4 + c] = *p++;
                    }
                }
        }
        else
        {
            if (end - p < 4 * width)
            {
                error = "truncated HDR data";
                return false;
            }
            std::memcpy(line.data(), p, size_t(width) * 4);
            p += size_t(width) * 4;
        }
        for (int x = 0; x < width; x++)
        {
            const uint8_t* e = &line[size_t(x) * 4];
            float f          = e[3] ? std::ldexp(1.0f, int(e[3]) - (128 + 8)) : 0.f;
            float* o         = &rgb[(size_t(y) * width + x) * 3];
            o[0] = e[0] * f, o[1] = e[1] * f, o[2] = e[2] * f;
        }
    }
    return true;
}

bool savePNG(const std::string& path, const uint8_t* rgba, int width, int height, size_t stride)
{
    std::vector<uint8_t> raw;
    raw.reserve(size_t(height) * (size_t(width) * 4 + 1));
    for (int y = 0; y < height; y++)
    {
        raw.push_back(0); // filter: none
        raw.insert(raw.end(), rgba + size_t(y) * stride, rgba + size_t(y) * stride + size_t(width) * 4);
    }
    // zlib stream of stored (uncompressed) deflate blocks.
    std::vector<uint8_t> z = { 0x78, 0x01 };
    uint32_t a = 1, b = 0;
    for (uint8_t v : raw)
    {
        a = (a + v) % 65521u;
        b = (b + a) % 65521u;
    }
    for (size_t off = 0; off < raw.size() || off == 0;)
    {
        size_t n  = std::min<size_t>(65535, raw.size() - off);
        bool last = off + n == raw.size();
        z.push_back(last ? 1 : 0);
        z.push_back(uint8_t(n & 0xff));
        z.push_back(uint8_t(n >> 8));
        z.push_back(uint8_t(~n & 0xff));
        z.push_back(uint8_t((~n >> 8) & 0xff));
        z.insert(z.end(), raw.begin() + off, raw.begin() + off + n);
        off += n;
        if (last)
            break;
    }
    uint32_t adler = (b << 16) | a;
    for (int s = 24; s >= 0; s -= 8)
        z.push_back(uint8_t(adler >> s));
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f)
        return false;
    auto put32 = [&](uint32_t v) {
        uint8_t be[4] = { uint8_t(v >> 24), uint8_t(v >> 16), uint8_t(v >> 8), uint8_t(v) };
        std::fwrite(be, 1, 4, f);
    };
    auto chunk = [&](const char* type, const std::vector<uint8_t>& body) {
        put32(uint32_t(body.size()));
        std::vector<uint8_t> tb(type, type + 4);
        tb.insert(tb.end(), body.begin(), body.end());
        std::fwrite(tb.data(), 1, tb.size(), f);
        put32(crc32(tb.data(), tb.size()) ^ 0xffffffffu);
    };
    const uint8_t sig[8] = { 0x89, 'P', 'N', 'G', 0x0d, 0x0a, 0x1a, 0x0a };
    std::fwrite(sig, 1, 8, f);
    std::vector<uint8_t> ihdr = { uint8_t(width >> 24), uint8_t(width >> 16), uint8_t(width >> 8), uint8_t(width),
        uint8_t(height >> 24), uint8_t(height >> 16), uint8_t(height >> 8), uint8_t(height), 8, 6, 0, 0, 0 };
    chunk("IHDR", ihdr);
    chunk("IDAT", z);
    chunk("IEND", {});
    bool ok = std::ferror(f) == 0;
    return std::fclose(f) == 0 && ok;
}

bool savePFM(const std::string& path, const float* rgba, int width, int height, size_t stride)
{
    FILE* f = std::fopen(path.c_str(), "wb");
    if (!f)
        return false;
    std::fprintf(f, "PF\n%d %d\n-1.0\n", width, height);
    std::vector<float> row(size_t(width) * 3);
    for (int y = height - 1; y >= 0; y--)
    {
        const float* src = reinterpret_cast<const float*>(reinterpret_cast<const uint8_t*>(rgba) + size_t(y) * stride);
        for (int x = 0; x < width; x++)
            for (int c = 0; c < 3; c++)
                row[size_t(x) * 3 + c] = src[size_t(x) * 4 + c];
        std::fwrite(row.data(), sizeof(float), row.size(), f);
    }
    bool ok = std::ferror(f) == 0;
    return std::fclose(f) == 0 && ok;
}

void fitCamera(const vec3& bmin, const vec3& bmax, const vec3& direction, float fovY, float aspect, vec3& eye,
    vec3& target)
{
    target = { 0.5f * (bmin[0] + bmax[0]), 0.5f * (bmin[1] + bmax[1]), 0.5f * (bmin[2] + bmax[2]) };
    // View basis of lookAt(target - direction, target, up (0, 1, 0)).
    auto unit = [](vec3 v) {
        float l = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        return vec3{ v[0] / l, v[1] / l, v[2] / l };
    };
    auto cross = [](const vec3& a, const vec3& b) {
        return vec3{ a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0] };
    };
    vec3 f = unit(direction);
    vec3 s = unit(cross(f, vec3{ 0.f, 1.f, 0.f }));
    vec3 u = cross(s, f);
    float lo[3] = { INFINITY, INFINITY, INFINITY }, hi[3] = { -INFINITY, -INFINITY, -INFINITY };
    for (int c = 0; c < 8; c++)
    {
        vec3 p = { (c & 1) ? bmax[0] : bmin[0], (c & 2) ? bmax[1] : bmin[1], (c & 4) ? bmax[2] : bmin[2] };
        float v[3];
        for (int k = 0; k < 3; k++)
        {
            const vec3& axis = k == 0 ? s : (k == 1 ? u : f);
            v[k] = axis[0] * p[0] + axis[1] * p[1] + axis[2] * p[2];
        }
        for (int k = 0; k < 3; k++)
        {
            lo[k] = std::min(lo[k], v[k]);
            hi[k] = std::max(hi[k], v[k]);
        }
    }
    float dims[3]   = { hi[0] - lo[0], hi[1] - lo[1], hi[2] - lo[2] };
    float boxAspect = dims[0] / dims[1];
    float halfFOV   = boxAspect > aspect ? std::atan(std::tan(fovY * 0.5f) * aspect) : fovY * 0.5f;
    float size      = boxAspect > aspect ? dims[0] : dims[1];
    float distance  = size / (2.0f * std::tan(halfFOV)) + dims[2] / 2.0f;
    eye = { target[0] - distance * f[0], target[1] - distance * f[1], target[2] - distance * f[2] };
}

} // namespace agb_aurora
