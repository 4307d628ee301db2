// aurora_gb300_loaders.hpp - scene and image I/O of the headless renderer (agb_render), after the
// Plasma application's batch path (Applications/Plasma/OBJLoader.cpp, Loaders.h, Camera.cpp):
// Wavefront OBJ + MTL files into an agb_aurora::IScene, Radiance HDR environment images, PNG /
// PFM output, and the camera fit to the scene bounds.
//
// The OBJ parse restates what the reference takes from tinyobjloader: v / vt / vn / f records
// (1-based or negative relative indices, polygons triangulated as a fan), a new shape at each
// `o` or `g` record, `usemtl` per face, `mtllib` material files; material defaults ior 1,
// dissolve 1, all colours 0.  The translation into Aurora objects follows OBJLoader.cpp:155-449.
#pragma once

#include <string>
#include <vector>

#include "aurora_gb300.hpp"

namespace agb_aurora
{

// What the reference gets from tinyobjloader.
struct ObjMaterial
{
    std::string name;
    float diffuse[3]       = { 0.f, 0.f, 0.f };
    float specular[3]      = { 0.f, 0.f, 0.f };
    float transmittance[3] = { 0.f, 0.f, 0.f };
    float emission[3]      = { 0.f, 0.f, 0.f };
    float ior              = 1.f;
    float dissolve         = 1.f;
    float roughness        = 0.f;
    float metallic         = 0.f;
    std::string diffuseTex, roughnessTex, emissiveTex, alphaTex, bumpTex, normalTex;
};
struct ObjIndex
{
    int position = -1, texcoord = -1, normal = -1; // 0-based, -1 when absent
};
struct ObjShape
{
    std::string name;
    std::vector<ObjIndex> indices;  // three per triangle
    std::vector<int> materialIds;   // one per triangle, -1 without usemtl
};
struct ObjData
{
    std::vector<float> positions, normals, texcoords;
    std::vector<ObjShape> shapes;
    std::vector<ObjMaterial> materials;
    std::string warnings;
};
// Parses OBJ text; `readFile` supplies material libraries by name (relative to the OBJ file).
AGB_CPP_API bool parseOBJ(const std::string& text,
    const std::function<bool(const std::string&, std::string&)>& readFile, ObjData& out,
    std::string& error);

// Scene data the loader keeps alive for the renderer's pull callbacks (Plasma's SceneContents).
struct SceneGeometryData
{
    std::vector<float> positions, normals, texCoords;
    std::vector<uint32_t> indices;
};
struct SceneInstanceData
{
    Path instance, geometry, material; // material empty: the renderer's default material
    mat4 transform = { 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1 }; // column-major
};
struct SceneMaterialData
{
    Path path;
    Properties properties;
};
// An image file a material refers to, handed to IScene::setImageFromFilePath.
struct SceneImageData
{
    Path path;
    std::string file;
    bool linearize = true;
};
// A camera of a glTF file (Plasma's SceneCamera, SceneContents.h:27-61).
struct SceneCamera
{
    enum Type
    {
        Perspective,
        Orthographic
    };
    Type type = Perspective;
    std::string name;
    mat4 viewMatrix = { 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1 }; // column-major
    float yfov = 0.f, aspectRatio = 0.f; // perspective
    float xmag = 0.f, ymag = 0.f;        // orthographic
    float znear = 0.f, zfar = 0.f;
};
struct SceneContents
{
    std::map<Path, SceneGeometryData> geometry;
    std::vector<SceneCamera> cameras;
    std::vector<SceneInstanceData> instances;
    std::vector<SceneMaterialData> materials;
    std::vector<SceneImageData> images;
    vec3 boundsMin = { 0.f, 0.f, 0.f }, boundsMax = { 0.f, 0.f, 0.f };
    uint32_t vertexCount = 0, triangleCount = 0;
    std::string warnings;
    void reset() { *this = SceneContents(); }
};
// The reference's translation of parsed OBJ data (OBJLoader.cpp:155-449): Standard Surface
// properties from the MTL values, unique (position, normal, texcoord) vertices per shape,
// normalised normals, flipped V, generated normals where the file has none, one instance per
// shape with the material of its first face.  Texture files (map_Kd and map_Ke decoded from
// sRGB, map_Pr, map_d and norm / bump linear; OBJLoader.cpp:176-227) become image paths
// `PlasmaImage/<file>:linearize:<0|1>` listed in contents.images, the file resolved beside the
// OBJ file; emission is 1 when there is an emission colour image.
AGB_CPP_API bool translateOBJ(const ObjData& obj, const std::string& filePath, SceneContents& contents);
// With this set, an OBJ material whose name has a .mtlx file beside the OBJ file takes that
// MaterialX document instead (OBJLoader.cpp:124-150, Plasma's --loadMtlXForObj); off by default.
AGB_CPP_API void loadMaterialXForOBJMaterials(bool enabled);
// loadOBJFile (OBJLoader.cpp:73-473): parse + translate + hand everything to the scene.
AGB_CPP_API bool loadOBJFile(IScene* scene, const std::string& filePath, SceneContents& contents);

// Hands loaded contents to a scene: materials, geometry descriptors that pull from `contents`
// (which must outlive the scene's use of them), instances with their transforms, bounds.
AGB_CPP_API void addContentsToScene(IScene* scene, SceneContents& contents);

// glTF 2.0 (.gltf with embedded or external buffers, .glb) after the reference's loader
// (Applications/Plasma/glTFLoader.cpp:26-436; the file parse restates what it takes from
// tinygltf): every scene's nodes, recursively, with matrix or TRS transforms accumulated from
// the parents; each TRIANGLES primitive with FLOAT positions becomes one geometry
// (`<file>:gltfGeom:<n>`) and one instance (`<file>:gltfInst:<n>`) with the node's world
// transform; NORMAL and TEXCOORD_0 when present (FLOAT), normals generated otherwise, unsigned
// 8/16/32-bit indices or a sequential list; one material per glTF material
// (`<file>:gltfMat:<i>`) with base_color, metalness and specular_roughness from
// pbrMetallicRoughness (glTF defaults 1, 1, 1); camera nodes collected with the inverse of the
// node's own transform as the view.  A node's AURORA_materials_materialX extension names a .mtlx
// file beside the glTF file that gives the node's material (`AURORA_mtlx:<file>`, read with
// materialXFileToProperties); when it cannot be read the glTF material is used, with a warning.
// With a null scene the contents are filled and no scene is touched.
AGB_CPP_API bool loadglTFFile(IScene* scene, const std::string& filePath, SceneContents& contents);
// Writes the contents' cameras as a glTF file of camera nodes (glTFLoader.cpp:438-492).
AGB_CPP_API bool saveglTFFile(const std::string& filePath, const SceneContents& contents);

// MaterialX (the reference generates shader code from the document, Source/MaterialX/
// MaterialGenerator.cpp:30-120 mapping standard_surface inputs to its material fields): here a
// document whose surface shader -- the surfaceshader input of its first surfacematerial, else its
// first standard_surface node -- is a standard_surface becomes the built-in material's
// properties, one per constant input (float, integer, boolean, color3 / vector3, the rgb of
// color4) under the input's name.  An image or tiledimage node (directly or as a node graph's
// output) feeding base_color, specular_roughness, emission_color or opacity becomes that
// texture: `<input>_image` = an image path for the file (relative paths against baseDirectory),
// listed in `images` with linearize for the srgb_texture colour space, uvtiling / uvoffset as the texture
// scale / offset.  Other connected inputs keep their defaults and other surface shaders are
// refused, each with a warning.
struct MaterialXImage
{
    std::string property; // e.g. base_color_image
    Path image;           // the image path the property names: MaterialXImage/<file>:linearize:<0|1>
    std::string file;
    bool linearize = false;
};
AGB_CPP_API bool materialXToProperties(const std::string& document, const std::string& baseDirectory,
    Properties& properties, std::string& warnings, std::vector<MaterialXImage>& images);
// Without a scene to load image files into: connected images are reported.
AGB_CPP_API bool materialXToProperties(const std::string& document, Properties& properties, std::string& warnings);
AGB_CPP_API bool materialXFileToProperties(const std::string& path, Properties& properties, std::string& warnings,
    std::vector<MaterialXImage>* images = nullptr);

// Angle-weighted smooth vertex normals (Foundation/Source/Geometry.cpp:29-99).
AGB_CPP_API void calculateNormals(size_t vertexCount, const float* positions, size_t triangleCount,
    const uint32_t* indices, float* normalsOut);

// PNG files to 8-bit RGBA, top row first (agb_image_io.cpp: zlib / DEFLATE and the scanline
// filters restated from RFC 1950 / 1951 and the PNG specification): grey, grey + alpha, RGB, RGBA
// and palette images at 1-16 bits, non-interlaced.
AGB_CPP_API bool decodePNG(const std::string& data, std::vector<uint8_t>& rgba, int& width, int& height,
    std::string& error);
AGB_CPP_API bool loadPNGFile(const std::string& path, std::vector<uint8_t>& rgba, int& width, int& height,
    std::string& error);

// Radiance RGBE (.hdr) image, flat or run-length encoded scanlines, to RGB floats top row first.
AGB_CPP_API bool loadHDRFile(const std::string& path, std::vector<float>& rgb, int& width, int& height,
    std::string& error);
AGB_CPP_API bool decodeHDR(const std::string& data, std::vector<float>& rgb, int& width, int& height,
    std::string& error);
// 8-bit RGBA PNG (stored deflate blocks) and little-endian PFM (RGB float, bottom row first).
AGB_CPP_API bool savePNG(const std::string& path, const uint8_t* rgba, int width, int height, size_t stride);
AGB_CPP_API bool savePFM(const std::string& path, const float* rgba, int width, int height, size_t stride);

// Camera::fit (Plasma/Camera.cpp:145-178): target = box centre, eye backed off along -direction
// until the box fills the vertical (or horizontal) field of view.
AGB_CPP_API void fitCamera(const vec3& boundsMin, const vec3& boundsMax, const vec3& direction,
    float fovYRadians, float aspect, vec3& eye, vec3& target);

} // namespace agb_aurora
