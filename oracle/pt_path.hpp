// Oracle (test infrastructure, never linked into the product): the path-level restatement.
//   Shaders/Random.slang:96-137          PCG2D random numbers
//   Shaders/RayTrace.slang:130-182       computeCameraRay
//   Shaders/RayTrace.slang:221-270       traceShadowRay (forced-opaque and transparent shadows)
//   Shaders/Geometry.slang:131-265       computeShadingData
//   Shaders/DefaultMaterial.slang:130-239 evaluateDefaultMaterial (textures, UV transforms)
//   Shaders/ShadeFunctions.slang:31-310  emission, distant light, environment MIS, next ray
//   Shaders/HitShaderEntryPoints.slang:35-486 closest hit incl. the material-layer loop
//       (DirectX branch of GlobalBufferAccessors.slang:60-127 for layer data)
//   Shaders/MainEntryPoints.slang:70-334, 355-426 ray-gen path loop and miss shader
//   Shaders/PathTracingCommon.slang:59-82 adjustRadiance
//   HGI/Shaders/Accumulation.glsl:14-34  running-mean accumulation
//   HGI/Shaders/PostProcessing.glsl:37-64 brightness, ACES, sRGB, alpha = 1
// The random numbers are always computed in FP32 (uint -> float), so the FP32 and FP64
// instantiations draw identical sample streams.
#pragma once

#include "pt_bsdf.hpp"
#include "pt_bvh.hpp"
#include "pt_env.hpp"
#include "pt_temporal.hpp"

namespace orc
{

struct Rng
{
    uint32_t x = 0, y = 0;
};

// Random.slang:96-108
inline Rng pcg2DInit(uint32_t sampleIndex, uint32_t screenWidth, uint32_t px, uint32_t py)
{
    Rng r;
    r.x = py * screenWidth + px;
    r.y = sampleIndex;
    return r;
}
// Random.slang:113-137
inline V2<float> random2Df(Rng& rng)
{
    uint32_t vx = rng.x, vy = rng.y;
    vx += vy * 1664525u;
    vy += vx * 1664525u;
    vx ^= vx >> 16u;
    vy ^= vy >> 16u;
    vx += vy * 1664525u;
    vy += vx * 1664525u;
    vx ^= vx >> 16u;
    vy ^= vy >> 16u;
    rng.x = vx;
    rng.y = vy;
    const float denom = float(0xFFFFFFFFu);
    return V2<float>(float(vx) / denom, float(vy) / denom);
}
// Note on the advance: pcg2D() returns the hashed pair and pcg2DNext2D() stores that pair back as
// the state (Random.slang:133), so the LCG step inside pcg2D is overwritten and the next draw hashes
// the previous output.

template <class T>
inline V2<T> random2D(Rng& rng)
{
    V2<float> r = random2Df(rng);
    return V2<T>(T(r.x), T(r.y));
}

struct Scene
{
    const Mesh* meshes               = nullptr;
    int32_t meshCount                = 0;
    const Instance* instances        = nullptr;
    int32_t instanceCount            = 0;
    const MaterialBlock* materials   = nullptr;
    int32_t materialCount            = 0;
    const MaterialTextures* materialTextures = nullptr; // may be null (no textures)
    const Image* images              = nullptr;
    int32_t imageCount               = 0;
    const EnvData* env               = nullptr;
    const Image* envLight            = nullptr;
    const Image* envBackground       = nullptr;
    const AliasEntry* envAlias       = nullptr;
    // Material node-graph programs (agb_material_graphs_set): material m runs
    // graphOps[graphFirst[m] .. + graphCount[m]); null when no material has one.
    const int32_t* graphFirst        = nullptr;
    const int32_t* graphCount        = nullptr;
    const agb_graph_op* graphOps     = nullptr;
    const float* graphConsts         = nullptr; // 4 per constant
};

// Ground plane: the layout of the C ABI's agb_ground_plane (the caller's IGroundPlane values,
// Aurora.h:780-806; PTGroundPlane.cpp:62-83).  enabled == 0: no ground plane.
struct GroundPlaneData
{
    int32_t enabled           = 0;
    float position[3]         = { 0.f, 0.f, 0.f };
    float normal[3]           = { 0.f, 1.f, 0.f };
    float shadowOpacity       = 1.f;
    float shadowColor[3]      = { 0.f, 0.f, 0.f };
    float reflectionOpacity   = 0.5f;
    float reflectionColor[3]  = { 0.5f, 0.5f, 0.5f };
    float reflectionRoughness = 0.1f;
};


// MaterialX's noise functions (its stdlib's mx_noise.glsl, after Open Shading Language): the
// lattice hash is Bob Jenkins' lookup3 final mix of the integer cell (a = b = c = 0xdeadbeef +
// 4 n + 13, plus the n coordinates); Perlin's improved noise takes gradients from the hash's low
// bits (8 directions in 2D, 12 edges in 3D), blends them with the fade 6t^5 - 15t^4 + 10t^3 and
// scales by 0.6616 (2D) / 0.9820 (3D); cell noise is the cell's hash / 0xffffffff.  T: float or
// double for the blend; the hash is 32-bit integer arithmetic either way.
template <class T>
struct MxNoise
{
    static uint32_t rotl(uint32_t x, int k) { return (x << k) | (x >> (32 - k)); }
    static uint32_t mix(uint32_t a, uint32_t b, uint32_t c)
    {
        c = (c ^ b) - rotl(b, 14);
        a = (a ^ c) - rotl(c, 11);
        b = (b ^ a) - rotl(a, 25);
        c = (c ^ b) - rotl(b, 16);
        a = (a ^ c) - rotl(c, 4);
        b = (b ^ a) - rotl(a, 14);
        c = (c ^ b) - rotl(b, 24);
        return c;
    }
    static uint32_t hash(int x, int y)
    {
        const uint32_t init = 0xdeadbeefu + 8u + 13u;
        return mix(init + uint32_t(x), init + uint32_t(y), init);
    }
    static uint32_t hash(int x, int y, int z)
    {
        const uint32_t init = 0xdeadbeefu + 12u + 13u;
        return mix(init + uint32_t(x), init + uint32_t(y), init + uint32_t(z));
    }
    static T fade(T t) { return t * t * t * (t * (t * T(6) - T(15)) + T(10)); }
    static T gradient(uint32_t h, T x, T y)
    {
        const bool low = (h & 7u) < 4u;
        const T a = low ? x : y, b = T(2) * (low ? y : x);
        return ((h & 1u) ? -a : a) + ((h & 2u) ? -b : b);
    }
    static T gradient(uint32_t h, T x, T y, T z)
    {
        h &= 15u;
        const T a = h < 8u ? x : y;
        const T b = h < 4u ? y : (h == 12u || h == 14u) ? x : z;
        return ((h & 1u) ? -a : a) + ((h & 2u) ? -b : b);
    }
    static T perlin2(T px, T py)
    {
        const int X = int(std::floor(px)), Y = int(std::floor(py));
        const T fx = px - T(X), fy = py - T(Y), u = fade(fx), v = fade(fy);
        const T g00 = gradient(hash(X, Y), fx, fy), g10 = gradient(hash(X + 1, Y), fx - T(1), fy);
        const T g01 = gradient(hash(X, Y + 1), fx, fy - T(1));
        const T g11 = gradient(hash(X + 1, Y + 1), fx - T(1), fy - T(1));
        const T iu = T(1) - u, iv = T(1) - v;
        return T(0.6616f) * (iv * (g00 * iu + g10 * u) + v * (g01 * iu + g11 * u));
    }
    static T perlin3(T px, T py, T pz)
    {
        const int X = int(std::floor(px)), Y = int(std::floor(py)), Z = int(std::floor(pz));
        const T fx = px - T(X), fy = py - T(Y), fz = pz - T(Z);
        const T u = fade(fx), v = fade(fy), w = fade(fz);
        T g[8];
        for (int k = 0; k < 8; k++)
        {
            const int dx = k & 1, dy = (k >> 1) & 1, dz = k >> 2;
            g[k] = gradient(hash(X + dx, Y + dy, Z + dz), dx ? fx - T(1) : fx, dy ? fy - T(1) : fy,
                dz ? fz - T(1) : fz);
        }
        const T iu = T(1) - u, iv = T(1) - v, iw = T(1) - w;
        return T(0.9820f) * (iw * (iv * (g[0] * iu + g[1] * u) + v * (g[2] * iu + g[3] * u)) +
                                w * (iv * (g[4] * iu + g[5] * u) + v * (g[6] * iu + g[7] * u)));
    }
    static T cell2(T px, T py)
    {
        return T(float(hash(int(std::floor(px)), int(std::floor(py))))) / T(float(0xffffffffu));
    }
    static T cell3(T px, T py, T pz)
    {
        return T(float(hash(int(std::floor(px)), int(std::floor(py)), int(std::floor(pz))))) / T(float(0xffffffffu));
    }
};

template <class T>
struct PathTracer
{
    using v2 = V2<T>;
    using v3 = V3<T>;
    using B  = BSDF<T>;
    using E  = Env<T>;

    const Scene* scene    = nullptr;
    const FrameData* frame = nullptr;
    Caster<T> caster;
    typename E::Scene env;
    uint32_t screenW = 0, screenH = 0;

    // Per-thread statistics (camera-path segments and shadow rays traced).
    struct Stats
    {
        uint64_t raysTraced = 0, shadowRaysTraced = 0;
    };
    static Stats& stats()
    {
        static thread_local Stats s;
        return s;
    }

    void init(const Scene* s, const FrameData* f, uint32_t w, uint32_t h, bool bruteForce = false)
    {
        scene   = s;
        frame   = f;
        screenW = w;
        screenH = h;
        caster.bruteForce = bruteForce;
        caster.build(s->meshes, s->meshCount, s->instances, s->instanceCount);
        env.data       = s->env;
        env.lightImage = s->envLight;
        env.background = s->envBackground;
        env.alias      = s->envAlias;
    }

    // The scene's ground plane and the tangent frame the host builds from its normal
    // (PTGroundPlane.cpp:23-28, in FP32 as the constant buffer holds it).
    GroundPlaneData ground;
    float groundTangent[3]   = { 1.f, 0.f, 0.f };
    float groundBitangent[3] = { 0.f, 0.f, 1.f };
    void setGroundPlane(const GroundPlaneData* g)
    {
        ground = g ? *g : GroundPlaneData{};
        if (!g)
        {
            ground.enabled = 0;
            return;
        }
        const float* n = ground.normal;
        float b[3]     = { 0.f, 1.f, 0.f };
        if (!(std::fabs(n[1]) < 0.999f))
        {
            b[0] = 1.f;
            b[1] = 0.f;
        }
        float t[3] = { b[1] * n[2] - b[2] * n[1], b[2] * n[0] - b[0] * n[2], b[0] * n[1] - b[1] * n[0] };
        float inv  = 1.f / std::sqrt(t[0] * t[0] + t[1] * t[1] + t[2] * t[2]);
        for (int k = 0; k < 3; k++)
            groundTangent[k] = t[k] * inv;
        const float* u     = groundTangent;
        groundBitangent[0] = n[1] * u[2] - n[2] * u[1];
        groundBitangent[1] = n[2] * u[0] - n[0] * u[2];
        groundBitangent[2] = n[0] * u[1] - n[1] * u[0];
    }

    // RayTrace.slang:130-182
    void computeCameraRay(uint32_t px, uint32_t py, Rng& rng, v3& origin, v3& direction) const
    {
        const FrameData& f = *frame;
        v2 sc{T(float(px)), T(float(py))};
        if (f.isTemporalJitterEnabled)
            sc = sc + v2(T(0.5f) + T(f.cameraJitter[0]), T(0.5f) + T(f.cameraJitter[1]));
        else
            sc = sc + random2D<T>(rng);
        v2 ndc(sc.x / T(float(screenW)), sc.y / T(float(screenH)));
        ndc         = v2(ndc.x * T(2) - T(1), ndc.y * T(2) - T(1));
        ndc.y       = -ndc.y;
        const float* m = f.cameraInvView;
        v3 right{T(m[0]), T(m[4]), T(m[8])};
        v3 up{T(m[1]), T(m[5]), T(m[9])};
        v3 front = -v3(T(m[2]), T(m[6]), T(m[10]));
        v3 eye{T(m[3]), T(m[7]), T(m[11])};
        v2 size{T(f.viewSize[0]) * T(0.5f), T(f.viewSize[1]) * T(0.5f)};
        v3 offset = right * (size.x * ndc.x) + up * (size.y * ndc.y);
        if (f.isOrthoProjection)
        {
            direction = front;
            origin    = eye + offset;
        }
        else
        {
            direction = normalize(front + offset);
            origin    = eye;
        }
        if (f.lensRadius > 0.f)
        {
            v3 focalPoint = origin + direction * T(f.focalDistance);
            v2 off        = B::sampleDisk(random2D<T>(rng), T(f.lensRadius));
            origin        = origin + right * off.x + up * off.y;
            direction     = normalize(focalPoint - origin);
        }
    }

    // Geometry.slang:131-148
    static v3 projectOnPlane(const v3& p, const v3& o, const v3& n) { return p - n * dot(p - o, n); }

    // Geometry.slang:152-265 (tangent from the up vector: HGI never reports tangents).
    ShadingData<T> computeShadingData(int32_t inst, uint32_t tri, T u, T v) const
    {
        const Instance& in = scene->instances[inst];
        const Mesh& m      = scene->meshes[in.mesh];
        ShadingData<T> sh;
        v3 bary{T(1) - u - v, u, v};
        sh.barycentrics = bary;
        uint32_t idx[3] = { m.indices[3 * size_t(tri)], m.indices[3 * size_t(tri) + 1],
            m.indices[3 * size_t(tri) + 2] };
        v3 pos[3], nrm[3];
        v3 gp(0), n(0);
        v2 uv{T(0), T(0)};
        for (int i = 0; i < 3; i++)
        {
            pos[i] = v3::from(m.positions + 3 * size_t(idx[i]));
            gp += pos[i] * bary[i];
            if (m.normals)
            {
                nrm[i] = v3::from(m.normals + 3 * size_t(idx[i]));
                n += nrm[i] * bary[i];
            }
            if (m.texcoords)
            {
                v2 t{T(m.texcoords[2 * size_t(idx[i])]), T(m.texcoords[2 * size_t(idx[i]) + 1])};
                uv = uv + t * bary[i];
            }
            sh.indices[i] = idx[i];
        }
        v3 objectNormal = normalize(m.normals ? n : cross(pos[1] - pos[0], pos[2] - pos[0]));
        v3 objectPosition = gp;
        if (m.normals)
        {
            v3 p0 = projectOnPlane(gp, pos[0], nrm[0]);
            v3 p1 = projectOnPlane(gp, pos[1], nrm[1]);
            v3 p2 = projectOnPlane(gp, pos[2], nrm[2]);
            v3 sp = p0 * bary.x + p1 * bary.y + p2 * bary.z;
            objectPosition = dot(sp - gp, n) > T(0) ? sp : gp;
        }
        Xform<T> x;
        for (int k = 0; k < 12; k++)
            x.m[k] = T(in.objectToWorld[k]);
        sh.position     = x.point(objectPosition);
        sh.geomPosition = x.point(gp);
        sh.normal       = normalize(x.vector(objectNormal));
        v3 up = std::fabs(sh.normal.y) < T(0.999f) ? v3(0, 1, 0) : v3(1, 0, 0);
        sh.tangent   = normalize(cross(sh.normal, up));
        sh.bitangent = cross(sh.normal, sh.tangent);
        sh.texCoord  = uv;
        return sh;
    }

    // DefaultMaterial.slang:88-105
    static v2 applyUVTransform(v2 uv, const float* pivot, const float* scale, float rotate,
        const float* offset)
    {
        v2 p{T(pivot[0]), T(pivot[1])};
        v2 sub = uv - p;
        v2 scaled(sub.x / T(scale[0]), sub.y / T(scale[1]));
        T r  = T(rotate) * (Consts<T>::PI / T(180));
        T sa = tsin(r), ca = tcos(r);
        v2 rot(ca * scaled.x + sa * scaled.y, -sa * scaled.x + ca * scaled.y);
        v2 tr(rot.x - T(offset[0]), rot.y - T(offset[1]));
        return tr + p;
    }

    bool sampleMaterialTexture(int32_t material, int slot, v2 uv, const float* pivot,
        const float* scale, float rotation, const float* offset, v3& rgb) const
    {
        if (!scene->materialTextures)
            return false;
        int32_t img = scene->materialTextures[material].image[slot];
        if (img < 0 || img >= scene->imageCount)
            return false;
        T a;
        E::sample(scene->images[img], applyUVTransform(uv, pivot, scale, rotation, offset), rgb, a);
        return true;
    }

    // The inverse of an instance's object-to-world transform as the host computes it for the
    // device: double precision, rounded to float.
    static void worldToObject(const float* m, float* out)
    {
        double a = m[0], b = m[1], c = m[2], d = m[4], e = m[5], f = m[6], g = m[8], h = m[9], i = m[10];
        double A = e * i - f * h, Bq = -(d * i - f * g), C = d * h - e * g;
        double det = a * A + b * Bq + c * C;
        double inv[9] = { A / det, -(b * i - c * h) / det, (b * f - c * e) / det, Bq / det,
            (a * i - c * g) / det, -(a * f - c * d) / det, C / det, -(a * h - b * g) / det,
            (a * e - b * d) / det };
        double tx = m[3], ty = m[7], tz = m[11];
        for (int r = 0; r < 3; r++)
        {
            out[4 * r + 0] = float(inv[3 * r + 0]);
            out[4 * r + 1] = float(inv[3 * r + 1]);
            out[4 * r + 2] = float(inv[3 * r + 2]);
            out[4 * r + 3] = float(-(inv[3 * r + 0] * tx + inv[3 * r + 1] * ty + inv[3 * r + 2] * tz));
        }
    }

    // A material's node-graph program over the hit (the operations documented with
    // agb_material_graphs_set), run after its constants and textures: writes the fields it drives.
    void runMaterialGraph(int32_t matIndex, const ShadingData<T>& sh, const Instance* inst, Material<T>& m,
        v3& materialNormal, bool& isGeneratedNormal) const
    {
        struct R4
        {
            T v[4];
        };
        R4 r[AGB_GRAPH_REGS];
        for (auto& q : r)
            q = R4{ { T(0), T(0), T(0), T(0) } };
        const int32_t first = scene->graphFirst[matIndex], count = scene->graphCount[matIndex];
        for (int32_t k = 0; k < count; k++)
        {
            const agb_graph_op& o = scene->graphOps[first + k];
            const R4 A = r[o.a], B = r[o.b], C = r[o.c], D = r[o.d];
            R4 v = A;
            auto each = [&](auto f) {
                for (int c = 0; c < 4; c++)
                    v.v[c] = f(A.v[c], B.v[c], C.v[c]);
            };
            switch (o.op)
            {
            case AGB_GOP_CONST:
                for (int c = 0; c < 4; c++)
                    v.v[c] = T(scene->graphConsts[4 * o.imm + c]);
                break;
            case AGB_GOP_INPUT:
            {
                v3 q(T(0));
                switch (o.imm)
                {
                case AGB_GIN_TEXCOORD: q = v3(sh.texCoord.x, sh.texCoord.y, T(0)); break;
                case AGB_GIN_POSITION_WORLD: q = sh.geomPosition; break;
                case AGB_GIN_POSITION_OBJECT:
                    if (inst)
                    {
                        float w[12];
                        worldToObject(inst->objectToWorld, w);
                        const v3& p = sh.geomPosition;
                        q = v3(T(w[0]) * p.x + T(w[1]) * p.y + T(w[2]) * p.z + T(w[3]),
                            T(w[4]) * p.x + T(w[5]) * p.y + T(w[6]) * p.z + T(w[7]),
                            T(w[8]) * p.x + T(w[9]) * p.y + T(w[10]) * p.z + T(w[11]));
                    }
                    else
                        q = sh.geomPosition;
                    break;
                case AGB_GIN_NORMAL_WORLD: q = sh.normal; break;
                case AGB_GIN_NORMAL_OBJECT:
                    if (inst)
                    {
                        const float* o2w = inst->objectToWorld;
                        const v3& n      = sh.normal;
                        q = normalize(v3(T(o2w[0]) * n.x + T(o2w[4]) * n.y + T(o2w[8]) * n.z,
                            T(o2w[1]) * n.x + T(o2w[5]) * n.y + T(o2w[9]) * n.z,
                            T(o2w[2]) * n.x + T(o2w[6]) * n.y + T(o2w[10]) * n.z));
                    }
                    else
                        q = sh.normal;
                    break;
                case AGB_GIN_TANGENT_WORLD: q = sh.tangent; break;
                case AGB_GIN_BITANGENT_WORLD: q = sh.bitangent; break;
                default: break;
                }
                v = R4{ { q.x, q.y, q.z, T(0) } };
                break;
            }
            case AGB_GOP_ADD: each([](T a, T b, T) { return a + b; }); break;
            case AGB_GOP_SUB: each([](T a, T b, T) { return a - b; }); break;
            case AGB_GOP_MUL: each([](T a, T b, T) { return a * b; }); break;
            case AGB_GOP_DIV: each([](T a, T b, T) { return a / b; }); break;
            case AGB_GOP_MIN: each([](T a, T b, T) { return std::fmin(a, b); }); break;
            case AGB_GOP_MAX: each([](T a, T b, T) { return std::fmax(a, b); }); break;
            case AGB_GOP_POW: each([](T a, T b, T) { return tpow(a, b); }); break;
            case AGB_GOP_MOD: each([](T a, T b, T) { return a - b * std::floor(a / b); }); break;
            case AGB_GOP_FLOOR: each([](T a, T, T) { return std::floor(a); }); break;
            case AGB_GOP_CEIL: each([](T a, T, T) { return std::ceil(a); }); break;
            case AGB_GOP_ABS: each([](T a, T, T) { return std::fabs(a); }); break;
            case AGB_GOP_SIN: each([](T a, T, T) { return tsin(a); }); break;
            case AGB_GOP_COS: each([](T a, T, T) { return tcos(a); }); break;
            case AGB_GOP_SQRT: each([](T a, T, T) { return std::sqrt(a); }); break;
            case AGB_GOP_SIGN: each([](T a, T, T) { return a > T(0) ? T(1) : a < T(0) ? T(-1) : T(0); }); break;
            case AGB_GOP_CLAMP: each([](T a, T b, T c) { return std::fmin(std::fmax(a, b), c); }); break;
            case AGB_GOP_MIX: each([](T a, T b, T c) { return b + c * (a - b); }); break;
            case AGB_GOP_DOT:
            case AGB_GOP_NORMALIZE:
            case AGB_GOP_LENGTH:
            {
                const R4& bb = o.op == AGB_GOP_DOT ? B : A;
                T d = T(0);
                for (int c = 0; c < 4 && c < o.d; c++)
                    d = c == 0 ? A.v[0] * bb.v[0] : d + A.v[c] * bb.v[c];
                if (o.op == AGB_GOP_DOT)
                    v = R4{ { d, d, d, d } };
                else
                {
                    const T len = std::sqrt(d);
                    if (o.op == AGB_GOP_LENGTH)
                        v = R4{ { len, len, len, len } };
                    else
                    {
                        v = R4{ { T(0), T(0), T(0), T(0) } };
                        for (int c = 0; c < 4 && c < o.d; c++)
                            v.v[c] = A.v[c] / len;
                    }
                }
                break;
            }
            case AGB_GOP_SWIZZLE:
                v = R4{ { A.v[o.imm & 3], A.v[(o.imm >> 2) & 3], A.v[(o.imm >> 4) & 3], A.v[(o.imm >> 6) & 3] } };
                break;
            case AGB_GOP_COMBINE: v = R4{ { A.v[0], B.v[0], C.v[0], D.v[0] } }; break;
            case AGB_GOP_SELECT:
            {
                const bool t = o.imm == 0 ? A.v[0] > B.v[0] : o.imm == 1 ? A.v[0] >= B.v[0] : A.v[0] == B.v[0];
                v            = t ? C : D;
                break;
            }
            case AGB_GOP_IMAGE:
            {
                v3 rgb;
                T alpha;
                E::sample(scene->images[o.imm], v2(A.v[0], A.v[1]), rgb, alpha);
                v = R4{ { rgb.x, rgb.y, rgb.z, alpha } };
                break;
            }
            case AGB_GOP_NORMALMAP:
            {
                v3 vv = v3(A.v[0], A.v[1], A.v[2]) * T(2) - v3(1);
                vv.x  = vv.x * B.v[0];
                vv.y  = vv.y * B.v[0];
                v3 Bn = normalize(cross(sh.normal, sh.tangent));
                v3 n  = normalize(sh.tangent * vv.x + Bn * vv.y + sh.normal * vv.z);
                v     = R4{ { n.x, n.y, n.z, T(0) } };
                break;
            }
            case AGB_GOP_NOISE:
            {
                const T q = o.imm == 0 ? MxNoise<T>::perlin2(A.v[0], A.v[1])
                    : o.imm == 1       ? MxNoise<T>::perlin3(A.v[0], A.v[1], A.v[2])
                    : o.imm == 2       ? MxNoise<T>::cell2(A.v[0], A.v[1])
                                       : MxNoise<T>::cell3(A.v[0], A.v[1], A.v[2]);
                v = R4{ { q, q, q, q } };
                break;
            }
            case AGB_GOP_OUTPUT:
                switch (o.imm)
                {
                case AGB_GOUT_BASE_COLOR: m.baseColor = v3(A.v[0], A.v[1], A.v[2]); break;
                case AGB_GOUT_SPECULAR_ROUGHNESS: m.specularRoughness = A.v[0]; break;
                case AGB_GOUT_COAT_ROUGHNESS: m.coatRoughness = A.v[0]; break;
                case AGB_GOUT_EMISSION_COLOR: m.emissionColor = v3(A.v[0], A.v[1], A.v[2]); break;
                case AGB_GOUT_OPACITY: m.opacity = v3(A.v[0], A.v[1], A.v[2]); break;
                case AGB_GOUT_NORMAL:
                    materialNormal    = v3(A.v[0], A.v[1], A.v[2]);
                    isGeneratedNormal = true;
                    break;
                default: break;
                }
                continue;
            default: break;
            }
            r[o.dst] = v;
        }
    }

    bool hasGraph(int32_t matIndex) const
    {
        return scene->graphFirst && scene->graphCount && scene->graphCount[matIndex] > 0;
    }

    // DefaultMaterial.slang:130-239; a node-graph program, when the material has one, runs last.
    Material<T> evaluateDefaultMaterial(int32_t matIndex, const ShadingData<T>& sh,
        v3& materialNormal, bool& isGeneratedNormal, const Instance* inst = nullptr) const
    {
        const MaterialBlock& b = scene->materials[matIndex];
        Material<T> m;
        m.base               = T(b.base);
        m.baseColor          = v3::from(b.baseColor);
        m.diffuseRoughness   = T(b.diffuseRoughness);
        m.metalness          = T(b.metalness);
        m.specular           = T(b.specular);
        m.specularColor      = v3::from(b.specularColor);
        m.specularRoughness  = T(b.specularRoughness);
        m.specularIOR        = T(b.specularIOR);
        m.specularAnisotropy = T(b.specularAnisotropy);
        m.specularRotation   = T(b.specularRotation);
        m.transmission       = T(b.transmission);
        m.transmissionColor  = v3::from(b.transmissionColor);
        m.subsurface         = T(b.subsurface);
        m.subsurfaceColor    = v3::from(b.subsurfaceColor);
        m.subsurfaceRadius   = v3::from(b.subsurfaceRadius);
        m.subsurfaceScale    = T(b.subsurfaceScale);
        m.subsurfaceAnisotropy = T(b.subsurfaceAnisotropy);
        m.sheen              = T(b.sheen);
        m.sheenColor         = v3::from(b.sheenColor);
        m.sheenRoughness     = T(b.sheenRoughness);
        m.coat               = T(b.coat);
        m.coatColor          = v3::from(b.coatColor);
        m.coatRoughness      = T(b.coatRoughness);
        m.coatAnisotropy     = T(b.coatAnisotropy);
        m.coatRotation       = T(b.coatRotation);
        m.coatIOR            = T(b.coatIOR);
        m.coatAffectColor    = T(b.coatAffectColor);
        m.coatAffectRoughness = T(b.coatAffectRoughness);
        m.emission           = T(b.emission);
        m.emissionColor      = v3::from(b.emissionColor);
        m.opacity            = v3::from(b.opacity);
        m.thinWalled         = b.thinWalled != 0;
        v3 rgb;
        if (b.hasBaseColorTex &&
            sampleMaterialTexture(matIndex, kTexBaseColor, sh.texCoord, b.baseColorTexPivot,
                b.baseColorTexScale, b.baseColorTexRotation, b.baseColorTexOffset, rgb))
            m.baseColor = rgb;
        if (b.hasSpecularRoughnessTex &&
            sampleMaterialTexture(matIndex, kTexSpecularRoughness, sh.texCoord,
                b.specularRoughnessTexPivot, b.specularRoughnessTexScale,
                b.specularRoughnessTexRotation, b.specularRoughnessTexOffset, rgb))
            m.specularRoughness = rgb.x;
        if (b.hasEmissionColorTex &&
            sampleMaterialTexture(matIndex, kTexEmission, sh.texCoord, b.emissionColorTexPivot,
                b.emissionColorTexScale, b.emissionColorTexRotation, b.emissionColorTexOffset, rgb))
            m.emissionColor = rgb;
        if (b.hasOpacityTex &&
            sampleMaterialTexture(matIndex, kTexOpacity, sh.texCoord, b.opacityTexPivot,
                b.opacityTexScale, b.opacityTexRotation, b.opacityTexOffset, rgb))
            m.opacity = rgb;
        isGeneratedNormal = false;
        if (b.hasNormalTex &&
            sampleMaterialTexture(matIndex, kTexNormal, sh.texCoord, b.normalTexPivot,
                b.normalTexScale, b.normalTexRotation, b.normalTexOffset, rgb))
        {
            v3 vv = rgb * T(2) - v3(1);
            v3 Bn = normalize(cross(sh.normal, sh.tangent));
            materialNormal    = normalize(sh.tangent * vv.x * T(1) + Bn * vv.y * T(1) + sh.normal * vv.z);
            isGeneratedNormal = true;
        }
        if (hasGraph(matIndex))
            runMaterialGraph(matIndex, sh, inst, m, materialNormal, isGeneratedNormal);
        m.metalColor = m.baseColor;
        return m;
    }

    // ShadeFunctions.slang:31-48
    static v3 shadeEmission(const Material<T>& m)
    {
        v3 blend = lerp(v3(1), m.coatColor, m.coat);
        return m.emissionColor * m.emission * blend;
    }

    // ShadeFunctions.slang:51-89
    static v3 shadeDirectionalLight(const DistantLight& l, const Material<T>& m,
        const ShadingData<T>& sh, const v3& V, Rng& rng, v3& shadowDir)
    {
        v2 random = random2D<T>(rng);
        v3 L      = B::sampleCone(random, v3::from(l.direction), T(l.cosRadius));
        v3 bsdf   = B::evaluateMaterial(m, sh, V, L);
        if (isBlack(bsdf))
        {
            shadowDir = v3(0);
            return v3(0);
        }
        v3 radiance = v3::from(l.colorAndIntensity) * T(l.colorAndIntensity[3]);
        shadowDir   = L;
        return radiance * bsdf;
    }

    struct MISOut
    {
        int lobeID              = NO_SECONDARY_RAY;
        bool emitsMaterial      = false;
        v3 materialResult       = v3(0);
        v3 materialDir          = v3(0);
        bool emitsLight         = false;
        v3 lightResult          = v3(0);
        v3 lightDir             = v3(0);
    };

    // ShadeFunctions.slang:135-259
    void shadeEnvironmentLightMIS(const Material<T>& m, const ShadingData<T>& sh, const v3& V,
        Rng& rng, MISOut& o, v2 pixel) const
    {
        v2 random = random2D<T>(rng);
        v3 L;
        T materialPDF;
        v3 bsdf = B::sampleMaterial(m, sh, V, random, L, materialPDF, o.lobeID);
        if (o.lobeID == TRANSMISSION_LOBE)
            return;
        v2 ss{T(float(screenW)), T(float(screenH))};
        v3 lightRadiance = E::evaluate(env, L, o.lobeID == TRANSMISSION_LOBE, pixel, ss);
        if (!isBlack(lightRadiance) && !isBlack(bsdf))
        {
            T lightPDF = scene->env->hasLightTex
                ? luminance(lightRadiance) / T(scene->env->lightTexLuminanceIntegral)
                : B::divPi(T(0.25f));
            T w = B::computeMISWeight(materialPDF, lightPDF);
            o.materialResult = lightRadiance * w * bsdf / materialPDF;
            o.materialDir    = L;
            o.emitsMaterial  = true;
        }
        T lightPDF;
        lightRadiance = E::sampleEnvironment(env, random, L, lightPDF);
        int evaluatedLobe;
        bsdf = B::evaluateMaterialAndPDF(m, sh, V, L, random, materialPDF, evaluatedLobe);
        if (!isBlack(lightRadiance) && !isBlack(bsdf))
        {
            T w           = B::computeMISWeight(lightPDF, materialPDF);
            o.lightResult = lightRadiance * w * bsdf / lightPDF;
            o.lightDir    = L;
            o.emitsLight  = true;
        }
    }

    // ShadeFunctions.slang:263-310
    static int setupIndirectLightRay(const Material<T>& m, const ShadingData<T>& sh, const v3& V,
        Rng& rng, v3& dir, v3& origin, v3& color)
    {
        v3 L;
        T pdf;
        int lobeID;
        v3 bsdf = B::sampleMaterial(m, sh, V, random2D<T>(rng), L, pdf, lobeID);
        if (isBlack(bsdf))
            return NO_SECONDARY_RAY;
        bool isTransmission = lobeID == TRANSMISSION_LOBE;
        origin = (dot(V, sh.normal) < T(0) || isTransmission) ? sh.geomPosition : sh.position;
        dir    = L;
        color  = bsdf / pdf;
        return lobeID;
    }

    // Opacity the transparent-shadow any-hit shader subtracts (HitShaderEntryPoints.slang:490-552).
    v3 shadowOpacity(const Hit& h) const
    {
        const Instance& in = scene->instances[h.inst];
        const MaterialBlock& b = scene->materials[in.material];
        bool hasOpacityImage = scene->materialTextures && b.hasOpacityTex &&
            scene->materialTextures[in.material].image[kTexOpacity] >= 0;
        bool opaque = b.opacity[0] == 1.f && b.opacity[1] == 1.f && b.opacity[2] == 1.f &&
            !hasOpacityImage && !hasGraph(in.material) && b.transmission == 0.f;
        if (opaque)
            return v3(1);
        ShadingData<T> sh = computeShadingData(h.inst, uint32_t(h.prim), T(h.u), T(h.v));
        v3 mn = sh.normal;
        bool gen;
        Material<T> m = evaluateDefaultMaterial(in.material, sh, mn, gen, &in);
        return m.opacity * (v3(1) - m.transmissionColor * m.transmission);
    }

    // RayTrace.slang:221-270
    v3 traceShadowRay(const v3& origin, const v3& L, int depth, int maxDepth) const
    {
        if (depth == maxDepth + 1)
            return v3(1);
        stats().shadowRaysTraced++;
        if (frame->isForceOpaqueShadowsEnabled)
            return caster.occluded(origin, L, Consts<T>::RAY_TMIN, T(INFINITY)) ? v3(0) : v3(1);
        // Transparent shadows: multiply (1 - opacity) over every intersection along the ray.
        v3 vis(1);
        T tmin = Consts<T>::RAY_TMIN;
        for (int guard = 0; guard < 4096; guard++)
        {
            Hit h;
            if (!caster.closest(origin, L, tmin, T(INFINITY), h))
                break;
            vis *= v3(1) - shadowOpacity(h);
            if (isBlack(vis))
                break;
            tmin = std::nextafter(T(h.t), T(INFINITY));
        }
        return vis;
    }

    struct Payload
    {
        Rng rng;
        v3 rayContribution = v3(1);
        v3 nextRayOrigin, nextRayDirection;
        v3 direct = v3(0), indirect = v3(0);
        bool isPrimaryRay = true, pathEnded = false, skipContribution = false, isInside = false;
        int rayType = CAMERA_RAY, nextRayType = 0, misLobeID = NO_SECONDARY_RAY, rayDepth = 0;
        T outputAlpha = T(0);
    };

    // Denoising AOVs of one sample per pixel (HitShaderEntryPoints.slang:149-233 for hits,
    // MainEntryPoints.slang:380-406 for misses, MainEntryPoints.slang:115-118 at ray generation):
    // view depth, guide normal + roughness, base colour + metalness and 2.5D motion, written while
    // the path is primary for sampleIndex == aovSample when the frame enables them.  Null pointers
    // or aovSample < 0 turn them off.
    float* aovDepth   = nullptr;
    float* aovNormal  = nullptr;
    float* aovAlbedo  = nullptr;
    float* aovMotion  = nullptr;
    int64_t aovSample = -1;
    // Added to the sample index that seeds the random streams (MainEntryPoints.slang:83).
    uint32_t seedOffset = 0;

    void writeHitAov(size_t i, const v3& rayOrigin, const v3& rayDirection, T t,
        const Material<T>& m, const v3& materialNormal) const
    {
        const FrameData& f = *frame;
        using TP           = Temporal<T>;
        v3 hw              = rayOrigin + rayDirection * t;
        T vz               = TP::viewZ(f.cameraInvView, hw);
        aovDepth[i]        = float(vz);
        v3 n               = normalize(materialNormal);
        T rough = m.specularRoughness > T(0.05f) ? m.specularRoughness : T(0.05f);
        float nr[4] = { float(n.x), float(n.y), float(n.z), float(rough) };
        float al[4] = { float(m.baseColor.x), float(m.baseColor.y), float(m.baseColor.z),
            float(m.metalness) };
        T mv[4];
        TP::motionVector(f.cameraViewProj, f.cameraViewProjPrev, f.cameraInvViewPrev, hw, vz,
            T(float(screenW)), T(float(screenH)), mv);
        for (int k = 0; k < 4; k++)
        {
            aovNormal[4 * i + k] = nr[k];
            aovAlbedo[4 * i + k] = al[k];
            aovMotion[4 * i + k] = float(mv[k]);
        }
    }
    void writeSkyAov(size_t i, const v3& rayDirection) const
    {
        const FrameData& f = *frame;
        aovDepth[i]        = f.skyViewZ;
        float nr[4] = { float(-rayDirection.x), float(-rayDirection.y), float(-rayDirection.z), 1.f };
        float al[4] = { 0.f, 0.f, 0.f, 0.1f };
        T mv[4];
        Temporal<T>::skyMotionVector(f.cameraViewProj, f.cameraViewProjPrev, rayDirection,
            T(float(screenW)), T(float(screenH)), mv);
        for (int k = 0; k < 4; k++)
        {
            aovNormal[4 * i + k] = nr[k];
            aovAlbedo[4 * i + k] = al[k];
            aovMotion[4 * i + k] = float(mv[k]);
        }
    }

    // sampleGGXSmithBRDF (BSDFCommon.slang:331-366) with anisotropy 0: roughnessToAlpha
    // (BSDFCommon.slang:194-204), the VNDF half-vector flipped for a lower-hemisphere view, the
    // reflected direction and its PDF, then evaluateGGXSmithBRDF (BSDFCommon.slang:310-327:
    // D G2 F / (4 |V.z| |L.z|), Schlick Fresnel BSDFCommon.slang:115-118, Smith G2 :231-240).
    static v3 sampleGGXSmithBRDF(const v3& V, const v3& f0, T roughness, v2 random, v3& L, T& pdf)
    {
        T a       = B::fmax_(T(0.0001f), roughness * roughness);
        v2 alpha(a * (T(1) + T(0)), a * (T(1) - T(0)));
        bool flip = V.z <= T(0);
        v3 H      = B::sampleGGXSmithVNDF(flip ? -V : V, alpha, random);
        H         = flip ? -H : H;
        L         = reflect(-V, H);
        T denom   = T(4) * dot(V, H);
        pdf       = B::evaluateGGXSmithVNDF(V, H, alpha) / denom;
        if (!(V.z * L.z > T(0)))
            return v3(0);
        v3 Hn = normalize(V + L);
        T D   = B::evaluateGGXNDF(Hn, alpha);
        T G2  = (dot(V, Hn) <= T(0) || dot(L, Hn) < T(0))
            ? T(0)
            : T(1) / (T(1) + B::lambda(V, alpha) + B::lambda(L, alpha));
        v3 F  = lerp(f0, v3(1), tpow(T(1) - dot(V, Hn), T(5)));
        return F * (D * G2) / (T(4) * std::fabs(V.z) * std::fabs(L.z));
    }

    // writeGroundPlaneGuideAOVs (GroundPlane.slang:197-233).
    void writeGroundAov(size_t i, const v3& pos) const
    {
        const FrameData& f = *frame;
        using TP           = Temporal<T>;
        T vz               = TP::viewZ(f.cameraInvView, pos);
        aovDepth[i]        = float(vz);
        const GroundPlaneData& g = ground;
        float rough = g.reflectionRoughness > 0.05f ? g.reflectionRoughness : 0.05f;
        float nr[4] = { g.normal[0], g.normal[1], g.normal[2], rough };
        float al[4] = { g.reflectionColor[0], g.reflectionColor[1], g.reflectionColor[2], 0.f };
        T mv[4];
        TP::motionVector(f.cameraViewProj, f.cameraViewProjPrev, f.cameraInvViewPrev, pos, vz,
            T(float(screenW)), T(float(screenH)), mv);
        for (int k = 0; k < 4; k++)
        {
            aovNormal[4 * i + k] = nr[k];
            aovAlbedo[4 * i + k] = al[k];
            aovMotion[4 * i + k] = float(mv[k]);
        }
    }

    // evaluateGroundPlane (GroundPlane.slang:236-289), run first by the closest-hit and miss
    // shaders: tCurrent is RayTCurrent() (the hit distance, infinity on a miss).  Returns true when
    // the ray was absorbed, i.e. continues as a matte reflection ray.
    bool evaluateGroundPlane(Payload& p, const v3& rayOrigin, const v3& rayDirection, T tCurrent,
        int64_t aovPixel) const
    {
        const GroundPlaneData& g = ground;
        if (!p.isPrimaryRay || !g.enabled)
            return false;
        // intersectGroundPlane (GroundPlane.slang:106-131).
        v3 N       = v3::from(g.normal);
        T planeDot = dot(rayDirection, N);
        if (planeDot >= T(0))
            return false;
        T dist = dot(v3::from(g.position) - rayOrigin, N) / planeDot;
        if (dist < T(0))
            return false;
        v3 pos = rayOrigin + rayDirection * dist;
        if (!(dist < tCurrent))
            return false;
        // setupGroundPlaneRay (GroundPlane.slang:136-193).
        v3 X = v3::from(groundTangent), Y = v3::from(groundBitangent);
        v3 color(1), nextDir(0), nextOrg(0);
        int rayType = CAMERA_RAY;
        bool chosen = false;
        if (g.reflectionOpacity > 0.f)
        {
            v3 transparency = v3(T(1) - T(g.reflectionOpacity));
            T Pr            = luminance(transparency);
            if (random2D<T>(p.rng).x >= Pr)
            {
                // setupMatteReflectionIndirectLightRay (GroundPlane.slang:26-67).
                v3 V = B::worldToTangent(-rayDirection, X, Y, N);
                v3 L;
                T pdf;
                v2 random = random2D<T>(p.rng);
                v3 bsdf   = sampleGGXSmithBRDF(V, v3::from(g.reflectionColor), T(g.reflectionRoughness),
                    random, L, pdf);
                bsdf *= std::fabs(L.z);
                if (isBlack(bsdf))
                {
                    rayType = NO_SECONDARY_RAY;
                    color   = v3(1);
                }
                else
                {
                    nextOrg = pos;
                    nextDir = B::tangentToWorld(L, X, Y, N);
                    color   = bsdf / pdf;
                    rayType = GROUND_PLANE_REFLECTION_RAY;
                }
                color *= T(g.reflectionOpacity) / (T(1) - Pr);
                chosen = true;
            }
            else
                color = transparency / Pr;
        }
        if (!chosen && g.shadowOpacity > 0.f)
        {
            // shadeMatteShadow (GroundPlane.slang:71-104): always an opaque shadow ray.
            v3 L;
            T pdf;
            E::sampleEnvironment(env, random2D<T>(p.rng), L, pdf);
            v3 shadowRGB(0);
            T shadowA = T(0);
            if (!(dot(L, N) < T(0)))
            {
                v3 vis(1);
                if (1 != frame->traceDepth + 1)
                {
                    stats().shadowRaysTraced++;
                    vis = caster.occluded(pos, L, Consts<T>::RAY_TMIN, T(INFINITY)) ? v3(0) : v3(1);
                }
                shadowRGB = v3::from(g.shadowColor);
                shadowA   = luminance(v3(1) - vis) * T(g.shadowOpacity);
            }
            color *= lerp(v3(1), shadowRGB, shadowA);
        }
        if (rayType == GROUND_PLANE_REFLECTION_RAY)
        {
            if (aovPixel >= 0)
                writeGroundAov(size_t(aovPixel), pos);
            p.nextRayType      = GROUND_PLANE_REFLECTION_RAY;
            p.rayContribution *= color;
            p.nextRayDirection = nextDir;
            p.nextRayOrigin    = nextOrg;
            p.isPrimaryRay     = false;
            return true;
        }
        p.rayContribution *= color;
        return false;
    }

    // Closest-hit shader (HitShaderEntryPoints.slang:35-486).  aovPixel: pixel index whose AOVs
    // this path writes, or -1.
    void closestHit(Payload& p, const v3& rayOrigin, const v3& rayDirection, const Hit& hit,
        v2 pixel, int64_t aovPixel) const
    {
        const FrameData& f = *frame;
        int maxTraceDepth  = f.traceDepth;
        v3 nextRayContribution(1);
        if (evaluateGroundPlane(p, rayOrigin, rayDirection, T(hit.t), aovPixel))
            return;
        v3 V              = -rayDirection;
        ShadingData<T> sh = computeShadingData(hit.inst, uint32_t(hit.prim), T(hit.u), T(hit.v));
        const Instance& in = scene->instances[hit.inst];
        bool hitLayer      = false;
        v2 baseLayerUV     = sh.texCoord;
        int layerCount     = in.layerCount;
        for (int li = layerCount; li >= 0; li--)
        {
            int32_t matIndex;
            if (li == 0)
            {
                matIndex    = in.material;
                sh.texCoord = baseLayerUV;
            }
            else
            {
                const Layer& L = in.layers[li - 1];
                matIndex       = L.material;
                v2 uv{T(0), T(0)};
                for (int i = 0; i < 3; i++)
                {
                    v2 t(T(L.texcoords[2 * size_t(sh.indices[i])]),
                        T(L.texcoords[2 * size_t(sh.indices[i]) + 1]));
                    uv = uv + t * sh.barycentrics[i];
                }
                sh.texCoord = uv;
            }
            bool isGeneratedNormal = false;
            v3 materialNormal      = sh.normal;
            Material<T> m = evaluateDefaultMaterial(matIndex, sh, materialNormal, isGeneratedNormal, &in);
            if (!p.isPrimaryRay && f.isPathRegularizationEnabled)
            {
                T fl = lerp(T(0.05f), lerp(T(0.05f), T(0.35f), T(f.pathRegularizationStrength)),
                    saturate(T(float(p.rayDepth)) / T(3)));
                m.specularRoughness = m.specularRoughness > fl ? m.specularRoughness : fl;
                m.coatRoughness     = m.coatRoughness > fl ? m.coatRoughness : fl;
            }
            if (p.isPrimaryRay && aovPixel >= 0)
                writeHitAov(size_t(aovPixel), rayOrigin, rayDirection, T(hit.t), m, materialNormal);
            v3 transparency = v3(1) - m.opacity;
            T P             = luminance(transparency);
            hitLayer        = random2D<T>(p.rng).x >= P;
            v3 dirShadowDir(0), dirColor(0);
            bool hasDirectionalLight = false;
            if (hitLayer)
            {
                if (isGeneratedNormal)
                {
                    sh.normal = materialNormal;
                    B::buildBasis(sh.normal, sh.tangent, sh.bitangent);
                }
                p.direct += shadeEmission(m);
                const LightData& lights = f.lights;
                bool evaluateAll = !f.isDenoisingAOVsEnabled && lights.distantLightCount > 1;
                if (evaluateAll)
                {
                    v3 o = dot(V, sh.normal) < T(0) ? sh.geomPosition : sh.position;
                    for (int li2 = 0; li2 < lights.distantLightCount; li2++)
                    {
                        if (lights.distantLights[li2].colorAndIntensity[3] <= 0.f)
                            continue;
                        v3 sd;
                        v3 r = shadeDirectionalLight(lights.distantLights[li2], m, sh, V, p.rng, sd);
                        if (isBlack(r))
                            continue;
                        v3 vis = traceShadowRay(o, sd, p.rayDepth, maxTraceDepth);
                        p.direct += vis * r;
                    }
                }
                else if (lights.distantLightCount > 0)
                {
                    float weights[4];
                    float total = 0.f;
                    for (int i = 0; i < lights.distantLightCount; i++)
                    {
                        const float* ci = lights.distantLights[i].colorAndIntensity;
                        float w = (ci[0] * 0.2125f + ci[1] * 0.7154f + ci[2] * 0.0721f) * ci[3];
                        weights[i] = w;
                        total += w;
                    }
                    int idx        = 0;
                    float selPdf   = 1.f / float(lights.distantLightCount);
                    if (total > 0.f)
                    {
                        float r   = random2Df(p.rng).x * total;
                        float cum = 0.f;
                        for (int i = 0; i < lights.distantLightCount; i++)
                        {
                            cum += weights[i];
                            if (r <= cum || i == lights.distantLightCount - 1)
                            {
                                idx    = i;
                                selPdf = weights[i] / total;
                                break;
                            }
                        }
                    }
                    else
                        idx = int(random2Df(p.rng).x * float(lights.distantLightCount));
                    if (lights.distantLights[idx].colorAndIntensity[3] > 0.f)
                    {
                        dirColor = shadeDirectionalLight(
                            lights.distantLights[idx], m, sh, V, p.rng, dirShadowDir);
                        dirColor /= T(selPdf > 1e-4f ? selPdf : 1e-4f);
                        hasDirectionalLight = true;
                    }
                }
                MISOut mis;
                shadeEnvironmentLightMIS(m, sh, V, p.rng, mis, pixel);
                p.rayContribution *= m.opacity / (T(1) - P);
                p.outputAlpha = (p.outputAlpha == T(0) && p.rayType == TRANSMISSION_LOBE) ? T(0) : T(1);
                p.nextRayType = setupIndirectLightRay(
                    m, sh, V, p.rng, p.nextRayDirection, p.nextRayOrigin, nextRayContribution);
                v3 so = dot(V, sh.normal) < T(0) ? sh.geomPosition : sh.position;
                if (hasDirectionalLight)
                {
                    v3 vis = traceShadowRay(so, dirShadowDir, p.rayDepth, maxTraceDepth);
                    p.direct += vis * dirColor;
                }
                if (mis.emitsLight || mis.emitsMaterial)
                {
                    v3 misResult(0);
                    if (mis.emitsMaterial)
                        misResult += traceShadowRay(so, mis.materialDir, p.rayDepth, maxTraceDepth) *
                            mis.materialResult;
                    if (mis.emitsLight)
                        misResult += traceShadowRay(so, mis.lightDir, p.rayDepth, maxTraceDepth) *
                            mis.lightResult;
                    p.misLobeID = mis.lobeID;
                    p.indirect  = misResult;
                }
                if (p.nextRayType == NO_SECONDARY_RAY)
                    p.pathEnded = true;
                p.isPrimaryRay = false;
                break;
            }
            else
                p.rayContribution *= transparency / P;
        }
        if (!hitLayer)
        {
            p.nextRayDirection = -V;
            p.nextRayOrigin    = sh.geomPosition;
            p.skipContribution = true;
            return;
        }
        if (p.nextRayType == TRANSMISSION_LOBE)
            p.isInside = !p.isInside;
        p.direct *= p.rayContribution;
        p.indirect *= p.rayContribution;
        p.rayContribution *= nextRayContribution;
        if (f.isRussianRouletteEnabled && p.rayDepth + 1 >= f.russianRouletteStartDepth)
        {
            v3 tp  = p.rayContribution;
            T mx   = tp.x > (tp.y > tp.z ? tp.y : tp.z) ? tp.x : (tp.y > tp.z ? tp.y : tp.z);
            T surv = clampT(mx, T(0.05f), T(1));
            if (random2D<T>(p.rng).x > surv)
                p.pathEnded = true;
            else
                p.rayContribution = p.rayContribution / surv;
        }
    }

    // PathTracingCommon.slang:59-82
    static void adjustRadiance(T maxLuminance, bool displayErrors, v3& radiance)
    {
        T lum = luminance(radiance);
        if (lum > maxLuminance)
            radiance *= maxLuminance / lum;
        bool isnan_ = std::isnan(radiance.x) || std::isnan(radiance.y) || std::isnan(radiance.z);
        bool isinf_ = std::isinf(radiance.x) || std::isinf(radiance.y) || std::isinf(radiance.z);
        if (isnan_)
            radiance = displayErrors ? v3(T(INFINITY), 0, 0) : v3(0);
        else if (isinf_)
            radiance = displayErrors ? v3(0, T(INFINITY), 0) : v3(0);
    }

    // Ray-generation shader (MainEntryPoints.slang:70-270) for one pixel sample.  Returns RGBA.
    void tracePath(uint32_t px, uint32_t py, uint32_t sampleIndex, T out[4]) const
    {
        const FrameData& f = *frame;
        int maxTraceDepth  = f.traceDepth;
        Payload p;
        p.rng = pcg2DInit(sampleIndex + seedOffset, screenW, px, py);
        v3 rayOrigin, rayDirection;
        computeCameraRay(px, py, p.rng, rayOrigin, rayDirection);
        v3 outDirect(0), outDiffuse(0), outGlossy(0);
        T outAlpha = T(0);
        v2 pixel{T(float(px)), T(float(py))};
        v2 ss{T(float(screenW)), T(float(screenH))};
        int64_t aovPixel = (f.isDenoisingAOVsEnabled && aovDepth && aovSample >= 0 &&
                               int64_t(sampleIndex) == aovSample)
            ? int64_t(py) * int64_t(screenW) + int64_t(px)
            : int64_t(-1);
        if (aovPixel >= 0)
            for (int k = 0; k < 4; k++)
                aovMotion[4 * size_t(aovPixel) + k] = 0.f;
        for (int rayDepth = 0; rayDepth <= maxTraceDepth && !p.pathEnded; rayDepth++)
        {
            if (rayDepth == maxTraceDepth)
            {
                bool bg = p.isPrimaryRay || p.rayType == TRANSMISSION_LOBE ||
                    p.rayType == GROUND_PLANE_REFLECTION_RAY;
                p.direct = E::evaluate(env, rayDirection, bg, pixel, ss);
                p.direct *= p.rayContribution;
                p.pathEnded = true;
            }
            else
            {
                T minT     = rayDepth == 0 ? T(0) : Consts<T>::RAY_TMIN;
                p.rayDepth = rayDepth;
                p.direct   = v3(0);
                p.indirect = v3(0);
                Hit hit;
                stats().raysTraced++;
                if (caster.closest(rayOrigin, rayDirection, minT, T(INFINITY), hit))
                    closestHit(p, rayOrigin, rayDirection, hit, pixel, aovPixel);
                else if (!evaluateGroundPlane(p, rayOrigin, rayDirection, T(INFINITY), aovPixel))
                {
                    bool bg = p.isPrimaryRay || p.rayType == TRANSMISSION_LOBE ||
                        p.rayType == GROUND_PLANE_REFLECTION_RAY;
                    if (bg)
                    {
                        p.direct = E::evaluate(env, rayDirection, true, pixel, ss);
                        p.direct *= p.rayContribution;
                    }
                    if (p.isPrimaryRay && aovPixel >= 0)
                        writeSkyAov(size_t(aovPixel), rayDirection);
                    p.pathEnded = true;
                }
                rayOrigin    = p.nextRayOrigin;
                rayDirection = p.nextRayDirection;
                outAlpha     = p.outputAlpha;
                if (p.skipContribution)
                {
                    p.skipContribution = false;
                    continue;
                }
            }
            if (rayDepth == 0)
            {
                p.isPrimaryRay = false;
                outDirect      = p.direct;
                if (p.misLobeID == DIFFUSE_LOBE)
                    outDiffuse = p.indirect;
                else
                    outGlossy = p.indirect;
            }
            else
            {
                v3 radiance = p.direct + p.indirect;
                if (f.indirectBounceClampScale > 0.f)
                    adjustRadiance(T(f.maxLuminance) * T(f.indirectBounceClampScale), false, radiance);
                if (p.rayType == DIFFUSE_LOBE)
                    outDiffuse += radiance;
                else
                    outGlossy += radiance;
            }
            p.rayType = p.nextRayType;
        }
        v3 fin = outDirect + outDiffuse + outGlossy;
        adjustRadiance(T(f.maxLuminance), f.isDisplayErrorsEnabled != 0, fin);
        out[0] = fin.x;
        out[1] = fin.y;
        out[2] = fin.z;
        out[3] = outAlpha;
    }
};

// Accumulation.glsl:14-34: mix(prev, cur, 1 / (n + 1)) for n > 0, else cur.
inline void accumulateRunningMean(float* acc, const float* cur, uint32_t sampleIndex)
{
    if (sampleIndex == 0)
    {
        for (int k = 0; k < 4; k++)
            acc[k] = cur[k];
        return;
    }
    float t = 1.0f / float(sampleIndex + 1);
    for (int k = 0; k < 4; k++)
        acc[k] = acc[k] * (1.0f - t) + cur[k] * t;
}

// PostProcessing.glsl:37-64
inline void postProcess(const float* acc, const float brightness[3], bool toneMap, bool gamma,
    float out[4])
{
    V3<float> c(acc[0] * brightness[0], acc[1] * brightness[1], acc[2] * brightness[2]);
    if (toneMap)
        c = toneMapACES(c);
    if (gamma)
        c = linearTosRGB(clamp3(c, 0.f, 1.f));
    out[0] = c.x;
    out[1] = c.y;
    out[2] = c.z;
    out[3] = 1.f;
}

} // namespace orc
