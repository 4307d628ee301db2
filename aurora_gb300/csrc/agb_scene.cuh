// Device-resident scene layout and the per-hit shading code that reads it:
//   images / texture sampling  (Texture2D.SampleLevel with repeat addressing),
//   environment evaluation and alias-table sampling (Shaders/Environment.slang:35-186),
//   computeShadingData (Shaders/Geometry.slang:131-265),
//   evaluateDefaultMaterial (Shaders/DefaultMaterial.slang:88-239).
#pragma once

#include "../../include/agb.h"
#include "agb_bsdf.cuh"

namespace agb
{

// ------------------------------------------------------------------------------ HBM layout
// BVH2 node, 64 bytes = four 128-bit loads.  Child refs: >= 0 interior node index; < 0 leaf with
// ~ref = (first << 3) | (count - 1), count <= 8 primitives.
struct __align__(16) BNode
{
    float4 c0xy; // child 0: lo.x hi.x lo.y hi.y
    float4 c1xy; // child 1: lo.x hi.x lo.y hi.y
    float4 cz;   // child 0 lo.z hi.z, child 1 lo.z hi.z
    int4 ref;    // child 0 ref, child 1 ref, unused, unused
};
static_assert(sizeof(BNode) == 64, "BNode is 64 bytes");

AGB_HD int32_t leafRef(uint32_t first, uint32_t count) { return ~int32_t((first << 3) | (count - 1)); }

struct DevImage
{
    const void* data; // RGBA8 or RGBA32F texels, rows top to bottom
    uint32_t width, height;
    int32_t format;   // AGB_FORMAT_RGBA8_UNORM or AGB_FORMAT_RGBA32F
    int32_t linear;
};

struct DevMesh
{
    const float* positions; // 3 per vertex
    const float* normals;   // 3 per vertex or null
    const float* texcoords; // 2 per vertex or null
    // 2 per vertex, the attributes one shading fetch needs: (position, normal.x), (normal.y,
    // normal.z, texcoord); normal and texcoord zero where the mesh has none.
    const float4* verts;
    const uint32_t* indices; // 3 per triangle
    const float4* tris;     // 3 per triangle in BVH leaf order: v0 (w = triangle id as int), v1, v2
    const BNode* nodes;
    uint32_t vertexCount, triangleCount;
    int32_t root;           // root ref
    int32_t depth;
};

struct DevLayer
{
    int32_t material;
    int32_t _pad;
    const float* texcoords; // 2 per base-mesh vertex
};

struct DevInstance
{
    float o2w[12];
    float w2o[12];
    int32_t mesh;
    int32_t material;
    int32_t layerCount;
    int32_t layerOffset; // into DevScene::layers
};

// Ground plane constants (the GroundPlane struct of GroundPlane.slang; PTGroundPlane.cpp:62-83):
// the caller's properties plus the tangent frame built from the normal.
struct DevGroundPlane
{
    int32_t enabled;
    float position[3];
    float normal[3];
    float tangent[3];
    float bitangent[3];
    float shadowOpacity;
    float shadowColor[3];
    float reflectionOpacity;
    float reflectionColor[3];
    float reflectionRoughness;
};

struct DevScene
{
    const DevMesh* meshes;
    const DevInstance* instances;
    const BNode* tlas;
    int32_t tlasRoot;
    int32_t instanceCount;
    const int32_t* tlasOrder; // instance index per TLAS leaf slot
    const agb_material* materials;
    const agb_material_textures* matTex; // may be null
    int32_t materialCount;
    int32_t imageCount;
    const DevImage* images;
    const DevLayer* layers;
    // Material node-graph programs (agb_material_graphs_set): per material (first op, op count),
    // null when no material has one.
    const int2* matGraph;
    const agb_graph_op* graphOps;
    const float4* graphConsts;
    // Environment.
    agb_environment_data env;
    DevImage envLight;        // data null when absent
    DevImage envBackground;   // data null when absent
    const agb_alias_entry* alias;
    DevGroundPlane ground;
};

// -------------------------------------------------------------------------- texture sampling
AGB_D float4 texel(const DevImage& im, int x, int y)
{
    int w = int(im.width), h = int(im.height);
    x     = x % w;
    x     = x < 0 ? x + w : x;
    y     = y % h;
    y     = y < 0 ? y + h : y;
    size_t i = size_t(y) * size_t(w) + size_t(x);
    if (im.format == AGB_FORMAT_RGBA8_UNORM)
    {
        uchar4 c = __ldg(static_cast<const uchar4*>(im.data) + i);
        return make_float4(float(c.x) / 255.f, float(c.y) / 255.f, float(c.z) / 255.f,
            float(c.w) / 255.f);
    }
    return __ldg(static_cast<const float4*>(im.data) + i);
}
AGB_D float4 lerp4(float4 a, float4 b, float t)
{
    return make_float4(a.x + t * (b.x - a.x), a.y + t * (b.y - a.y), a.z + t * (b.z - a.z),
        a.w + t * (b.w - a.w));
}
// SampleLevel(uv, 0) with repeat addressing; texel centres at (i + 0.5) / size.
AGB_D float4 sampleImage(const DevImage& im, v2 uv)
{
    float fw = float(im.width), fh = float(im.height);
    if (!im.linear)
        return texel(im, int(floorf(uv.x * fw)), int(floorf(uv.y * fh)));
    float x  = uv.x * fw - 0.5f;
    float y  = uv.y * fh - 0.5f;
    float x0 = floorf(x), y0 = floorf(y);
    float fx = x - x0, fy = y - y0;
    int ix = int(x0), iy = int(y0);
    float4 a = lerp4(texel(im, ix, iy), texel(im, ix + 1, iy), fx);
    float4 b = lerp4(texel(im, ix, iy + 1), texel(im, ix + 1, iy + 1), fx);
    return lerp4(a, b, fy);
}

// --------------------------------------------------------------------------- environment
AGB_D v2 dirToLatLong(v3 d)
{
    return v2{ ((agb_fm::atan2(d.x, -d.z) * 1.0f) / kPi) * 0.5f + 0.5f,
        ((-agb_fm::asin(d.y)) * 1.0f) / kPi + 0.5f };
}
AGB_D v3 latLongToDir(v2 uv)
{
    float phi   = (uv.x + 0.25f) * 2.f * kPi;
    float theta = uv.y * kPi;
    float sp, cp, st, ct;
    agb_fm::sincos(phi, &sp, &cp);
    agb_fm::sincos(theta, &st, &ct);
    return v3{ cp * st, ct, sp * st };
}
AGB_D v3 mulDir(const float* m, v3 d)
{
    return v3{ m[0] * d.x + m[1] * d.y + m[2] * d.z + m[3] * 0.f,
        m[4] * d.x + m[5] * d.y + m[6] * d.z + m[7] * 0.f,
        m[8] * d.x + m[9] * d.y + m[10] * d.z + m[11] * 0.f };
}
// Environment.slang:98-133.  pixel / screen are used only with background_use_screen.
AGB_DN v3 evaluateEnvironment(const DevScene& s, v3 dir, bool asBackground, v2 pixel, v2 screen)
{
    const agb_environment_data& c = s.env;
    if (asBackground)
    {
        v2 uv = c.background_use_screen ? v2{ pixel.x / screen.x, pixel.y / screen.y }
                                        : dirToLatLong(normalize(mulDir(c.background_transform, dir)));
        if (c.has_background_tex && s.envBackground.data)
        {
            float4 t = sampleImage(s.envBackground, uv);
            return v3{ t.x, t.y, t.z };
        }
        return lerp3(ld3(c.background_top), ld3(c.background_bottom), uv.y);
    }
    v2 uv = dirToLatLong(normalize(mulDir(c.light_transform, dir)));
    if (c.has_light_tex && s.envLight.data)
    {
        float4 t = sampleImage(s.envLight, uv);
        return v3{ t.x, t.y, t.z };
    }
    return lerp3(ld3(c.light_top), ld3(c.light_bottom), uv.y);
}
// Environment.slang:137-186
AGB_DN v3 sampleEnvironment(const DevScene& s, v2 r, v3& L, float& pdf)
{
    const agb_environment_data& c = s.env;
    if (c.has_light_tex && s.envLight.data)
    {
        uint32_t w = s.envLight.width, h = s.envLight.height, count = w * h;
        uint32_t index = uint32_t(float(count) * r.x);
        index          = index < count - 1 ? index : count - 1;
        float4 e       = __ldg(reinterpret_cast<const float4*>(s.alias) + index);
        if (e.y < r.y)
        {
            index = __float_as_uint(e.x);
            e     = __ldg(reinterpret_cast<const float4*>(s.alias) + index);
        }
        pdf        = e.z;
        uint32_t x = index % w, y = index / w;
        L = latLongToDir(v2{ (float(x) + 0.5f) / float(w), (float(y) + 0.5f) / float(h) });
        L = normalize(mulDir(c.light_transform_inv, L));
        float4 t = texel(s.envLight, int(x), int(y));
        return v3{ t.x, t.y, t.z };
    }
    L     = sampleUniformDirection(r, pdf);
    L     = normalize(mulDir(c.light_transform_inv, L));
    v2 uv = dirToLatLong(L);
    return lerp3(ld3(c.light_top), ld3(c.light_bottom), uv.y);
}

// ------------------------------------------------------------------------------ shading data
struct Shading
{
    v3 N, X, Y;         // world normal, tangent, bitangent
    v3 position;        // shadow-terminator shading position (world)
    v3 geomPosition;    // geometric hit position (world)
    v2 uv;
    uint32_t idx[3];
    v3 bary;
};

AGB_D v3 xfPoint(const float* m, v3 p)
{
    return v3{ m[0] * p.x + m[1] * p.y + m[2] * p.z + m[3],
        m[4] * p.x + m[5] * p.y + m[6] * p.z + m[7],
        m[8] * p.x + m[9] * p.y + m[10] * p.z + m[11] };
}
AGB_D v3 xfVector(const float* m, v3 v)
{
    return v3{ m[0] * v.x + m[1] * v.y + m[2] * v.z, m[4] * v.x + m[5] * v.y + m[6] * v.z,
        m[8] * v.x + m[9] * v.y + m[10] * v.z };
}
AGB_D v3 projectOnPlane(v3 p, v3 o, v3 n) { return p - n * dot(p - o, n); }

// Geometry.slang:152-265, tangent from the up vector (HGI reports no tangents).
AGB_D Shading computeShading(const DevScene& s, const DevInstance& in, uint32_t tri, float u, float v)
{
    const DevMesh& m = s.meshes[in.mesh];
    Shading sh;
    sh.bary = v3{ 1.f - u - v, u, v };
    uint3 id = make_uint3(__ldg(m.indices + 3 * size_t(tri)), __ldg(m.indices + 3 * size_t(tri) + 1),
        __ldg(m.indices + 3 * size_t(tri) + 2));
    sh.idx[0] = id.x;
    sh.idx[1] = id.y;
    sh.idx[2] = id.z;
    v3 p[3], nn[3];
    v3 gp = splat(0.f), n = splat(0.f);
    v2 uv = v2{ 0.f, 0.f };
    float b[3] = { sh.bary.x, sh.bary.y, sh.bary.z };
#pragma unroll
    for (int i = 0; i < 3; i++)
    {
        // One 32-byte vertex record (two 16-byte loads of one sector) instead of eight scalar
        // gathers from three arrays.
        const float4 va = __ldg(m.verts + 2 * size_t(sh.idx[i])), vb = __ldg(m.verts + 2 * size_t(sh.idx[i]) + 1);
        p[i] = v3{ va.x, va.y, va.z };
        gp += p[i] * b[i];
        if (m.normals)
        {
            nn[i] = v3{ va.w, vb.x, vb.y };
            n += nn[i] * b[i];
        }
        if (m.texcoords)
        {
            v2 t = v2{ vb.z, vb.w };
            uv = uv + t * b[i];
        }
    }
    v3 on = normalize(m.normals ? n : cross(p[1] - p[0], p[2] - p[0]));
    v3 op = gp;
    if (m.normals)
    {
        v3 sp = projectOnPlane(gp, p[0], nn[0]) * b[0] + projectOnPlane(gp, p[1], nn[1]) * b[1] +
            projectOnPlane(gp, p[2], nn[2]) * b[2];
        op = dot(sp - gp, n) > 0.f ? sp : gp;
    }
    sh.position     = xfPoint(in.o2w, op);
    sh.geomPosition = xfPoint(in.o2w, gp);
    sh.N            = normalize(xfVector(in.o2w, on));
    v3 up           = fabsf(sh.N.y) < 0.999f ? v3{ 0.f, 1.f, 0.f } : v3{ 1.f, 0.f, 0.f };
    sh.X            = normalize(cross(sh.N, up));
    sh.Y            = cross(sh.N, sh.X);
    sh.uv           = uv;
    return sh;
}

// DefaultMaterial.slang:88-105
AGB_D v2 uvTransform(v2 uv, const float* pivot, const float* scale, float rotate, const float* offset)
{
    v2 sub = v2{ uv.x - pivot[0], uv.y - pivot[1] };
    v2 sc  = v2{ sub.x / scale[0], sub.y / scale[1] };
    float r = rotate * (kPi / 180.f);
    float sa, ca;
    agb_fm::sincos(r, &sa, &ca);
    v2 rot = v2{ ca * sc.x + sa * sc.y, -sa * sc.x + ca * sc.y };
    return v2{ (rot.x - offset[0]) + pivot[0], (rot.y - offset[1]) + pivot[1] };
}

AGB_D bool materialTexture(const DevScene& s, int32_t mat, int slot, v2 uv, const float* pivot,
    const float* scale, float rotation, const float* offset, v3& rgb)
{
    if (!s.matTex)
        return false;
    int32_t img = s.matTex[mat].image[slot];
    if (img < 0 || img >= s.imageCount)
        return false;
    float4 t = sampleImage(s.images[img], uvTransform(uv, pivot, scale, rotation, offset));
    rgb      = v3{ t.x, t.y, t.z };
    return true;
}

// MaterialX's noise functions (stdlib genglsl mx_noise.glsl, after Open Shading Language's noise):
// Bob Jenkins' lookup3 "final" mix of the lattice point (seeded 0xdeadbeef + 4 n + 13 for n
// coordinates) as the hash; Perlin's improved noise (gradients from the hash's low bits, fade
// 6t^5 - 15t^4 + 10t^3, bi- / trilinear blend) scaled by 0.6616 in 2D and 0.9820 in 3D; cell noise
// = the cell's hash / 0xffffffff.
namespace mxNoise
{
AGB_D uint32_t rotl(uint32_t x, int k) { return (x << k) | (x >> (32 - k)); }
AGB_D uint32_t final3(uint32_t a, uint32_t b, uint32_t c)
{
    c ^= b;
    c -= rotl(b, 14);
    a ^= c;
    a -= rotl(c, 11);
    b ^= a;
    b -= rotl(a, 25);
    c ^= b;
    c -= rotl(b, 16);
    a ^= c;
    a -= rotl(c, 4);
    b ^= a;
    b -= rotl(a, 14);
    c ^= b;
    c -= rotl(b, 24);
    return c;
}
AGB_D uint32_t hash2(int x, int y)
{
    const uint32_t s = 0xdeadbeefu + (2u << 2) + 13u;
    return final3(s + uint32_t(x), s + uint32_t(y), s);
}
AGB_D uint32_t hash3(int x, int y, int z)
{
    const uint32_t s = 0xdeadbeefu + (3u << 2) + 13u;
    return final3(s + uint32_t(x), s + uint32_t(y), s + uint32_t(z));
}
AGB_D float fade(float t) { return t * t * t * (t * (t * 6.f - 15.f) + 10.f); }
AGB_D float negIf(float v, bool n) { return n ? -v : v; }
AGB_D float grad2(uint32_t h, float x, float y)
{
    h &= 7u;
    const float u = h < 4u ? x : y;
    const float v = 2.f * (h < 4u ? y : x);
    return negIf(u, h & 1u) + negIf(v, h & 2u);
}
AGB_D float grad3(uint32_t h, float x, float y, float z)
{
    h &= 15u;
    const float u = h < 8u ? x : y;
    const float v = h < 4u ? y : (h == 12u || h == 14u) ? x : z;
    return negIf(u, h & 1u) + negIf(v, h & 2u);
}
AGB_D float perlin2(float px, float py)
{
    const int X = int(floorf(px)), Y = int(floorf(py));
    const float fx = px - float(X), fy = py - float(Y);
    const float u = fade(fx), v = fade(fy);
    const float v0 = grad2(hash2(X, Y), fx, fy), v1 = grad2(hash2(X + 1, Y), fx - 1.f, fy);
    const float v2 = grad2(hash2(X, Y + 1), fx, fy - 1.f), v3 = grad2(hash2(X + 1, Y + 1), fx - 1.f, fy - 1.f);
    const float s1 = 1.f - u, t1 = 1.f - v;
    return 0.6616f * (t1 * (v0 * s1 + v1 * u) + v * (v2 * s1 + v3 * u));
}
AGB_D float perlin3(float px, float py, float pz)
{
    const int X = int(floorf(px)), Y = int(floorf(py)), Z = int(floorf(pz));
    const float fx = px - float(X), fy = py - float(Y), fz = pz - float(Z);
    const float u = fade(fx), v = fade(fy), w = fade(fz);
    const float v0 = grad3(hash3(X, Y, Z), fx, fy, fz), v1 = grad3(hash3(X + 1, Y, Z), fx - 1.f, fy, fz);
    const float v2 = grad3(hash3(X, Y + 1, Z), fx, fy - 1.f, fz);
    const float v3 = grad3(hash3(X + 1, Y + 1, Z), fx - 1.f, fy - 1.f, fz);
    const float v4 = grad3(hash3(X, Y, Z + 1), fx, fy, fz - 1.f);
    const float v5 = grad3(hash3(X + 1, Y, Z + 1), fx - 1.f, fy, fz - 1.f);
    const float v6 = grad3(hash3(X, Y + 1, Z + 1), fx, fy - 1.f, fz - 1.f);
    const float v7 = grad3(hash3(X + 1, Y + 1, Z + 1), fx - 1.f, fy - 1.f, fz - 1.f);
    const float s1 = 1.f - u, t1 = 1.f - v, r1 = 1.f - w;
    return 0.9820f * (r1 * (t1 * (v0 * s1 + v1 * u) + v * (v2 * s1 + v3 * u)) +
                         w * (t1 * (v4 * s1 + v5 * u) + v * (v6 * s1 + v7 * u)));
}
AGB_D float cell2(float px, float py) { return float(hash2(int(floorf(px)), int(floorf(py)))) / float(0xffffffffu); }
AGB_D float cell3(float px, float py, float pz)
{
    return float(hash3(int(floorf(px)), int(floorf(py)), int(floorf(pz)))) / float(0xffffffffu);
}
} // namespace mxNoise

// A material's node-graph program (the operations of agb_material_graphs_set) over the hit:
// writes the fields it drives into m / materialNormal.  Out of line, registers in local memory: it
// runs only for materials that have a program.
static __device__ __noinline__ void runMaterialGraph(const DevScene& s, int2 prog, const Shading& sh,
    const DevInstance* inst, Mat& m, v3& materialNormal, bool& generatedNormal)
{
    float4 r[AGB_GRAPH_REGS];
    for (int i = 0; i < AGB_GRAPH_REGS; i++)
        r[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int k = 0; k < prog.y; k++)
    {
        const agb_graph_op o = s.graphOps[prog.x + k];
        const float4 A = r[o.a], B = r[o.b], C = r[o.c], D = r[o.d];
        float4 v = A;
        switch (o.op)
        {
        case AGB_GOP_CONST: v = __ldg(s.graphConsts + o.imm); break;
        case AGB_GOP_INPUT:
        {
            v3 q = v3{ 0.f, 0.f, 0.f };
            switch (o.imm)
            {
            case AGB_GIN_TEXCOORD: q = v3{ sh.uv.x, sh.uv.y, 0.f }; break;
            case AGB_GIN_POSITION_WORLD: q = sh.geomPosition; break;
            case AGB_GIN_POSITION_OBJECT: q = inst ? xfPoint(inst->w2o, sh.geomPosition) : sh.geomPosition; break;
            case AGB_GIN_NORMAL_WORLD: q = sh.N; break;
            case AGB_GIN_NORMAL_OBJECT:
                // Normals go back to object space with the transpose of the object-to-world matrix.
                q = inst ? normalize(v3{ inst->o2w[0] * sh.N.x + inst->o2w[4] * sh.N.y + inst->o2w[8] * sh.N.z,
                               inst->o2w[1] * sh.N.x + inst->o2w[5] * sh.N.y + inst->o2w[9] * sh.N.z,
                               inst->o2w[2] * sh.N.x + inst->o2w[6] * sh.N.y + inst->o2w[10] * sh.N.z })
                         : sh.N;
                break;
            case AGB_GIN_TANGENT_WORLD: q = sh.X; break;
            case AGB_GIN_BITANGENT_WORLD: q = sh.Y; break;
            default: break;
            }
            v = make_float4(q.x, q.y, q.z, 0.f);
            break;
        }
        case AGB_GOP_ADD: v = make_float4(A.x + B.x, A.y + B.y, A.z + B.z, A.w + B.w); break;
        case AGB_GOP_SUB: v = make_float4(A.x - B.x, A.y - B.y, A.z - B.z, A.w - B.w); break;
        case AGB_GOP_MUL: v = make_float4(A.x * B.x, A.y * B.y, A.z * B.z, A.w * B.w); break;
        case AGB_GOP_DIV: v = make_float4(A.x / B.x, A.y / B.y, A.z / B.z, A.w / B.w); break;
        case AGB_GOP_MIN: v = make_float4(fminf(A.x, B.x), fminf(A.y, B.y), fminf(A.z, B.z), fminf(A.w, B.w)); break;
        case AGB_GOP_MAX: v = make_float4(fmaxf(A.x, B.x), fmaxf(A.y, B.y), fmaxf(A.z, B.z), fmaxf(A.w, B.w)); break;
        case AGB_GOP_POW:
            v = make_float4(agb_fm::pow(A.x, B.x), agb_fm::pow(A.y, B.y), agb_fm::pow(A.z, B.z), agb_fm::pow(A.w, B.w));
            break;
        case AGB_GOP_MOD:
            v = make_float4(A.x - B.x * floorf(A.x / B.x), A.y - B.y * floorf(A.y / B.y),
                A.z - B.z * floorf(A.z / B.z), A.w - B.w * floorf(A.w / B.w));
            break;
        case AGB_GOP_FLOOR: v = make_float4(floorf(A.x), floorf(A.y), floorf(A.z), floorf(A.w)); break;
        case AGB_GOP_CEIL: v = make_float4(ceilf(A.x), ceilf(A.y), ceilf(A.z), ceilf(A.w)); break;
        case AGB_GOP_ABS: v = make_float4(fabsf(A.x), fabsf(A.y), fabsf(A.z), fabsf(A.w)); break;
        case AGB_GOP_SIN:
            v = make_float4(agb_fm::sin(A.x), agb_fm::sin(A.y), agb_fm::sin(A.z), agb_fm::sin(A.w));
            break;
        case AGB_GOP_COS:
            v = make_float4(agb_fm::cos(A.x), agb_fm::cos(A.y), agb_fm::cos(A.z), agb_fm::cos(A.w));
            break;
        case AGB_GOP_SQRT: v = make_float4(sqrtf(A.x), sqrtf(A.y), sqrtf(A.z), sqrtf(A.w)); break;
        case AGB_GOP_SIGN:
            v = make_float4(A.x > 0.f ? 1.f : A.x < 0.f ? -1.f : 0.f, A.y > 0.f ? 1.f : A.y < 0.f ? -1.f : 0.f,
                A.z > 0.f ? 1.f : A.z < 0.f ? -1.f : 0.f, A.w > 0.f ? 1.f : A.w < 0.f ? -1.f : 0.f);
            break;
        case AGB_GOP_CLAMP:
            v = make_float4(fminf(fmaxf(A.x, B.x), C.x), fminf(fmaxf(A.y, B.y), C.y), fminf(fmaxf(A.z, B.z), C.z),
                fminf(fmaxf(A.w, B.w), C.w));
            break;
        case AGB_GOP_MIX:
            v = make_float4(B.x + C.x * (A.x - B.x), B.y + C.y * (A.y - B.y), B.z + C.z * (A.z - B.z),
                B.w + C.w * (A.w - B.w));
            break;
        case AGB_GOP_DOT:
        case AGB_GOP_NORMALIZE:
        case AGB_GOP_LENGTH:
        {
            const float* a = &A.x;
            const float* b = o.op == AGB_GOP_DOT ? &B.x : &A.x;
            float d = 0.f;
            for (int c = 0; c < 4 && c < o.d; c++)
                d = c == 0 ? a[0] * b[0] : d + a[c] * b[c];
            if (o.op == AGB_GOP_DOT)
                v = make_float4(d, d, d, d);
            else
            {
                const float len = sqrtf(d);
                if (o.op == AGB_GOP_LENGTH)
                    v = make_float4(len, len, len, len);
                else
                {
                    float out[4] = { 0.f, 0.f, 0.f, 0.f };
                    for (int c = 0; c < 4 && c < o.d; c++)
                        out[c] = a[c] / len;
                    v = make_float4(out[0], out[1], out[2], out[3]);
                }
            }
            break;
        }
        case AGB_GOP_SWIZZLE:
        {
            const float a[4] = { A.x, A.y, A.z, A.w };
            v = make_float4(a[o.imm & 3], a[(o.imm >> 2) & 3], a[(o.imm >> 4) & 3], a[(o.imm >> 6) & 3]);
            break;
        }
        case AGB_GOP_COMBINE: v = make_float4(A.x, B.x, C.x, D.x); break;
        case AGB_GOP_SELECT:
        {
            const bool t = o.imm == 0 ? A.x > B.x : o.imm == 1 ? A.x >= B.x : A.x == B.x;
            v            = t ? C : D;
            break;
        }
        case AGB_GOP_IMAGE:
            v = o.imm < s.imageCount ? sampleImage(s.images[o.imm], v2{ A.x, A.y }) : make_float4(0.f, 0.f, 0.f, 0.f);
            break;
        case AGB_GOP_NORMALMAP:
        {
            v3 vv = v3{ A.x, A.y, A.z } * 2.f - splat(1.f);
            vv.x  = vv.x * B.x;
            vv.y  = vv.y * B.x;
            v3 Bn = normalize(cross(sh.N, sh.X));
            v3 n  = normalize(sh.X * vv.x + Bn * vv.y + sh.N * vv.z);
            v     = make_float4(n.x, n.y, n.z, 0.f);
            break;
        }
        case AGB_GOP_NOISE:
        {
            const float q = o.imm == 0 ? mxNoise::perlin2(A.x, A.y)
                : o.imm == 1           ? mxNoise::perlin3(A.x, A.y, A.z)
                : o.imm == 2           ? mxNoise::cell2(A.x, A.y)
                                       : mxNoise::cell3(A.x, A.y, A.z);
            v = make_float4(q, q, q, q);
            break;
        }
        case AGB_GOP_OUTPUT:
            switch (o.imm)
            {
            case AGB_GOUT_BASE_COLOR: m.baseColor = v3{ A.x, A.y, A.z }; break;
            case AGB_GOUT_SPECULAR_ROUGHNESS: m.specularRoughness = A.x; break;
            case AGB_GOUT_COAT_ROUGHNESS: m.coatRoughness = A.x; break;
            case AGB_GOUT_EMISSION_COLOR: m.emissionColor = v3{ A.x, A.y, A.z }; break;
            case AGB_GOUT_OPACITY: m.opacity = v3{ A.x, A.y, A.z }; break;
            case AGB_GOUT_NORMAL:
                materialNormal  = v3{ A.x, A.y, A.z };
                generatedNormal = true;
                break;
            default: break;
            }
            continue;
        default: break;
        }
        r[o.dst] = v;
    }
}

// DefaultMaterial.slang:130-239; a node-graph program, when the material has one, runs last
// (kGraphs: the shading kernel's variant for scenes with programs; the variant without them
// carries no trace of the check).
template <bool kGraphs>
AGB_D Mat loadMaterial(const DevScene& s, int32_t mi, const Shading& sh, v3& materialNormal,
    bool& generatedNormal, const DevInstance* inst = nullptr)
{
    const agb_material& b = s.materials[mi];
    Mat m;
    m.b                 = &b;
    m.baseColor         = ldg3(b.base_color);
    m.specularRoughness = __ldg(&b.specular_roughness);
    m.coatRoughness     = __ldg(&b.coat_roughness);
    m.emissionColor     = ldg3(b.emission_color);
    m.opacity           = ldg3(b.opacity);
    v3 rgb;
    if (b.has_base_color_image &&
        materialTexture(s, mi, AGB_TEX_BASE_COLOR, sh.uv, b.base_color_image_pivot,
            b.base_color_image_scale, b.base_color_image_rotation, b.base_color_image_offset, rgb))
        m.baseColor = rgb;
    if (b.has_specular_roughness_image &&
        materialTexture(s, mi, AGB_TEX_SPECULAR_ROUGHNESS, sh.uv, b.specular_roughness_image_pivot,
            b.specular_roughness_image_scale, b.specular_roughness_image_rotation,
            b.specular_roughness_image_offset, rgb))
        m.specularRoughness = rgb.x;
    if (b.has_emission_color_image &&
        materialTexture(s, mi, AGB_TEX_EMISSION, sh.uv, b.emission_color_image_pivot,
            b.emission_color_image_scale, b.emission_color_image_rotation,
            b.emission_color_image_offset, rgb))
        m.emissionColor = rgb;
    if (b.has_opacity_image &&
        materialTexture(s, mi, AGB_TEX_OPACITY, sh.uv, b.opacity_image_pivot, b.opacity_image_scale,
            b.opacity_image_rotation, b.opacity_image_offset, rgb))
        m.opacity = rgb;
    generatedNormal = false;
    if (b.has_normal_image &&
        materialTexture(s, mi, AGB_TEX_NORMAL, sh.uv, b.normal_image_pivot, b.normal_image_scale,
            b.normal_image_rotation, b.normal_image_offset, rgb))
    {
        v3 vv  = rgb * 2.f - splat(1.f);
        v3 Bn  = normalize(cross(sh.N, sh.X));
        materialNormal  = normalize(sh.X * vv.x * 1.f + Bn * vv.y * 1.f + sh.N * vv.z);
        generatedNormal = true;
    }
    if (kGraphs && s.matGraph)
    {
        const int2 prog = __ldg(s.matGraph + mi);
        if (prog.y > 0)
            runMaterialGraph(s, prog, sh, inst, m, materialNormal, generatedNormal);
    }
    return m;
}

} // namespace agb
