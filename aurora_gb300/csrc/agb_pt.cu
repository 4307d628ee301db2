// Wavefront path-tracing kernels.  One wave traces `samples` sample indices for every pixel; the
// host (agb_render.cu) launches, per wave:
//   k_camera                                   RayGenShader prologue (MainEntryPoints.slang:70-121)
//   per bounce b < traceDepth:
//     k_trace_closest   closest-hit rays        TraceRay (RayTrace.slang:185-210)
//     k_shade           hit / miss shading      InstanceClosestHitShader + InstanceMissShader
//                                               (HitShaderEntryPoints.slang:35-486,
//                                                MainEntryPoints.slang:355-426)
//     k_trace_shadow    shadow rays             traceShadowRay (RayTrace.slang:221-270)
//     k_trace_shadow_transparent  the same with transparent shadows (any-hit opacity,
//                                               HitShaderEntryPoints.slang:490-552)
//     k_resolve         visibility x pending contributions, RayGen accumulation
//                                               (HitShaderEntryPoints.slang:394-467,
//                                                MainEntryPoints.slang:160-243)
//   k_shade (depth limit) environment at rayDepth == traceDepth (MainEntryPoints.slang:127-138)
//   k_finalize          adjustRadiance + accumulation (PathTracingCommon.slang:59-82,
//                                               HGI/Shaders/Accumulation.glsl:14-34)
// Shading arithmetic is compiled without multiply-add contraction (see the build flags) so that
// FP32 results follow the reference's operation order.
#include "agb_kernels.h"
#include "agb_temporal.cuh"

namespace agb
{

__device__ __forceinline__ unsigned long long* statPtr(const WaveBuffers& wb, int k)
{
    return wb.stats + k;
}

// ------------------------------------------------------------------------------ camera rays
// RayTrace.slang:130-182
__device__ void cameraRay(const agb_frame_data& f, uint32_t px, uint32_t py, uint32_t W,
    uint32_t H, Rng& rng, v3& o, v3& d)
{
    v2 sc = v2{ float(px), float(py) };
    if (f.is_temporal_jitter_enabled)
        sc = sc + v2{ 0.5f + f.camera_jitter[0], 0.5f + f.camera_jitter[1] };
    else
        sc = sc + random2D(rng);
    v2 ndc = v2{ sc.x / float(W), sc.y / float(H) };
    ndc    = v2{ ndc.x * 2.f - 1.f, ndc.y * 2.f - 1.f };
    ndc.y  = -ndc.y;
    const float* m = f.camera_inv_view;
    v3 right = v3{ m[0], m[4], m[8] };
    v3 up    = v3{ m[1], m[5], m[9] };
    v3 front = -v3{ m[2], m[6], m[10] };
    v3 eye   = v3{ m[3], m[7], m[11] };
    float sx = f.view_size[0] * 0.5f, sy = f.view_size[1] * 0.5f;
    v3 off   = right * (sx * ndc.x) + up * (sy * ndc.y);
    if (f.is_ortho_projection)
    {
        d = front;
        o = eye + off;
    }
    else
    {
        d = normalize(front + off);
        o = eye;
    }
    if (f.lens_radius > 0.f)
    {
        v3 focal = o + d * f.focal_distance;
        v2 lo    = sampleDisk(random2D(rng), f.lens_radius);
        o        = o + right * lo.x + up * lo.y;
        d        = normalize(focal - o);
    }
}

template <bool kBatch>
__global__ void k_camera(agb_frame_data f, WaveParams wp, WaveBuffers wb, BatchTables bt)
{
    uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < wp.paths; p += stride)
    {
        uint32_t r = 0, local = p;
        uint32_t pixels = wp.pixels, width = wp.width, height = wp.height, sampleBase = wp.sampleBase;
        uint32_t seedOffset = wp.seedOffset, aovSample = wp.aovSample;
        float4* aovMotion = wb.aovMotion;
        if constexpr (kBatch)
        {
            r                     = batchRequestOfPath(bt, p);
            const BatchRequest& q = bt.req[r];
            local      = p - q.pathOffset;
            pixels     = q.pixels;
            width      = q.width;
            height     = q.height;
            sampleBase = q.sampleBase;
            seedOffset = q.seedOffset;
            aovSample  = q.aovSample;
            aovMotion  = q.aovMotion;
            bt.pathReq[p] = uint16_t(r);
        }
        const agb_frame_data& F = kBatch ? bt.frames[r] : f;
        uint32_t samples = kBatch ? bt.req[r].samples : wp.samples;
        uint32_t pixel   = pathPixel(local, pixels, samples);
        uint32_t k       = pathSample(local, pixels, samples);
        uint32_t px = pixel % width, py = pixel / width;
        Rng rng     = rngInit(sampleBase + k + seedOffset, width, px, py);
        v3 o, d;
        cameraRay(F, px, py, width, height, rng, o, d);
        wb.rayOrg[0][p]  = make_float4(o.x, o.y, o.z, 0.f);
        wb.rayDir[0][p]  = make_float4(d.x, d.y, d.z, __int_as_float(0x7f800000));
        wb.rayPath[0][p] = p;
        wb.rng[p]        = make_uint2(rng.x, rng.y);
        wb.contrib[p]    = make_float4(1.f, 1.f, 1.f, 0.f);
        wb.flags[p] = PF_PRIMARY | (uint32_t(CAMERA_RAY) << PF_RAYTYPE_SHIFT) |
            (uint32_t(NO_SECONDARY_RAY) << PF_MISLOBE_SHIFT);
        if (sampleBase + k == aovSample)
            aovMotion[pixel] = make_float4(0.f, 0.f, 0.f, 0.f); // MainEntryPoints.slang:115-118
        float4 z = make_float4(0.f, 0.f, 0.f, 0.f);
        wb.outDirect[p]    = z;
        wb.outDiffuse[p]   = z;
        wb.outGlossy[p]    = z;
        wb.lastIndirect[p] = z;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0)
        wb.counters[0] = wp.paths;
}

// --------------------------------------------------------------------------------- tracing
extern __shared__ int32_t g_stack[];

struct QueueRayLoader
{
    const float4* org;
    const float4* dir;
    AGB_D void operator()(uint32_t i, v3& o, v3& d, float& tmin, float& tmax) const
    {
        float4 o4 = org[i], d4 = dir[i];
        o    = v3{ o4.x, o4.y, o4.z };
        d    = v3{ d4.x, d4.y, d4.z };
        tmin = o4.w;
        tmax = d4.w;
    }
};
struct HitWriter
{
    float4* tuv;
    int32_t* inst;
    AGB_D void operator()(uint32_t i, bool hit, const RayHit& h) const
    {
        tuv[i]  = make_float4(hit ? h.t : -1.f, h.u, h.v, __int_as_float(h.prim));
        inst[i] = hit ? h.inst : -1;
    }
};
// Batched waves: the TLAS root of the ray's scene, or kDone for a ray whose request has reached
// its trace depth (k_shade handles it as the depth-limit segment without its hit).
struct BatchQueueRayLoader : QueueRayLoader
{
    const uint32_t* rayPath;
    const uint16_t* pathReq;
    const BatchRequest* req;
    int bounce;
    AGB_D int32_t root(uint32_t i) const
    {
        const BatchRequest& q = req[pathReq[rayPath[i]]];
        return q.traceDepth <= bounce ? kDone : q.tlasRoot;
    }
};
struct ShadowLoader
{
    const uint32_t* tag;
    const float4* org;
    const float4* dir;
    AGB_D void operator()(uint32_t i, v3& o, v3& d, float& tmin, float& tmax) const
    {
        uint32_t t = tag[i];
        uint32_t p = t >> 3, k = t & 7u;
        float4 o4 = org[p];
        float4 d4 = dir[size_t(p) * kMaxShadowSlots + k];
        o    = v3{ o4.x, o4.y, o4.z };
        d    = v3{ d4.x, d4.y, d4.z };
        tmin = kRayTMin;
        tmax = __int_as_float(0x7f800000);
    }
};
struct BatchShadowLoader : ShadowLoader
{
    const uint16_t* pathReq;
    const BatchRequest* req;
    AGB_D int32_t root(uint32_t i) const { return req[pathReq[tag[i] >> 3]].tlasRoot; }
};
struct OcclusionWriter
{
    const uint32_t* tag;
    uint32_t* occluded;
    AGB_D void operator()(uint32_t i, bool hit, const RayHit&) const
    {
        if (hit)
        {
            uint32_t t = tag[i];
            atomicOr(occluded + (t >> 3), 1u << (t & 7u));
        }
    }
};

// Transparent shadows (is_force_opaque_shadows_enabled = 0): the any-hit shader of
// HitShaderEntryPoints.slang:490-552 multiplies the ray's visibility by 1 - opacity at every
// surface it crosses and ends the ray once it is black.  Here the hits are taken nearest first,
// each by a closest-hit traversal from just beyond the previous one, so the product has one
// order; at most kMaxShadowHits are taken.
constexpr int kMaxShadowHits = 4096;

// Opacity the any-hit shader takes from a hit: the instance's material opacity x (1 -
// transmission x transmission colour), 1 for an opaque material without an opacity texture.
AGB_DN v3 shadowOpacity(const DevScene& s, const RayHit& h)
{
    const DevInstance& in = s.instances[h.inst];
    const agb_material& b = s.materials[in.material];
    bool hasOpacityImage  = s.matTex && b.has_opacity_image && s.matTex[in.material].image[AGB_TEX_OPACITY] >= 0;
    // A node-graph program may drive the opacity: such a material is never taken as opaque here.
    bool hasGraph = s.matGraph && s.matGraph[in.material].y > 0;
    if (b.opacity[0] == 1.f && b.opacity[1] == 1.f && b.opacity[2] == 1.f && !hasOpacityImage && !hasGraph &&
        b.transmission == 0.f)
        return splat(1.f);
    Shading sh = computeShading(s, in, uint32_t(h.prim), h.u, h.v);
    v3 mn      = sh.N;
    bool gen;
    Mat m = loadMaterial<true>(s, in.material, sh, mn, gen, &in);
    return m.opacity * (splat(1.f) - m.transmissionColor() * m.transmission());
}

// Shadow rays of the transparent mode; `vis` (one float4 per shadow ray: running visibility, hits
// taken) reuses the shading-point buffer, which is free while shadow rays are traced.
struct TransparentShadowLoader
{
    ShadowLoader rays;
    float4* vis;
    AGB_D void operator()(uint32_t i, v3& o, v3& d, float& tmin, float& tmax) const
    {
        rays(i, o, d, tmin, tmax);
        vis[i] = make_float4(1.f, 1.f, 1.f, __int_as_float(0));
    }
};
struct BatchTransparentShadowLoader : TransparentShadowLoader
{
    const uint16_t* pathReq;
    const BatchRequest* req;
    AGB_D int32_t root(uint32_t i) const { return req[pathReq[rays.tag[i] >> 3]].tlasRoot; }
};
struct TransparentShadowWriter
{
    static constexpr bool kRestart = true;
    const uint32_t* tag;
    float4* vis;
    float4* pendSlot;
    // Returns false (trace on from the new tmin) while the ray is not blocked.
    AGB_D bool operator()(const DevScene& s, uint32_t i, bool hit, const RayHit& h, float& tmin) const
    {
        float4 v4 = vis[i];
        v3 v      = v3{ v4.x, v4.y, v4.z };
        if (hit)
        {
            v         = v * (splat(1.f) - shadowOpacity(s, h));
            int taken = __float_as_int(v4.w) + 1;
            if (!isBlack(v) && taken < kMaxShadowHits)
            {
                vis[i] = make_float4(v.x, v.y, v.z, __int_as_float(taken));
                tmin   = nextafterf(h.t, __int_as_float(0x7f800000));
                return false;
            }
        }
        // The slot's pending contribution times the visibility (traceShadowRay(...) * result);
        // its occlusion bit stays clear.
        uint32_t t = tag[i];
        float4* ps = pendSlot + size_t(t >> 3) * kMaxShadowSlots + (t & 7u);
        float4 c   = *ps;
        *ps        = make_float4(v.x * c.x, v.y * c.y, v.z * c.z, c.w);
        return true;
    }
};

template <bool kCount, bool kBatch>
__global__ void __launch_bounds__(kTraceBlock, kTraceBlocksPerSM) k_trace_closest(DevScene s, WaveBuffers wb,
    int bounce, int cur, BatchTables bt)
{
    uint32_t n      = wb.counters[bounce * kCounterStride + CNT_RAYS];
    TraceCounters c = { 0, 0 };
    bool overflow   = false;
    QueueRayLoader rays{ wb.rayOrg[cur], wb.rayDir[cur] };
    if constexpr (kBatch)
        persistentTrace<false, kCount>(s, n, wb.counters + bounce * kCounterStride + CNT_CLOSEST_WORK,
            BatchQueueRayLoader{ rays, wb.rayPath[cur], bt.pathReq, bt.req, bounce },
            HitWriter{ wb.hitTUV, wb.hitInst }, g_stack + threadIdx.x, kTraceBlock, c, overflow);
    else
        persistentTrace<false, kCount>(s, n, wb.counters + bounce * kCounterStride + CNT_CLOSEST_WORK, rays,
            HitWriter{ wb.hitTUV, wb.hitInst }, g_stack + threadIdx.x, kTraceBlock, c, overflow);
    if (kCount)
    {
        atomicAdd(statPtr(wb, 2), c.nodes);
        atomicAdd(statPtr(wb, 3), c.tris);
    }
    if (overflow)
        atomicAdd(statPtr(wb, 4), 1ull);
}

// Opaque shadow rays of the bounce's counter block: the shading's (CNT_SHADOW / CNT_SHADOW_WORK)
// or the ground plane's (CNT_GROUND_SHADOW / CNT_GROUND_WORK).
template <bool kCount, bool kBatch>
__global__ void __launch_bounds__(kTraceBlock, kTraceBlocksPerSM) k_trace_shadow(DevScene s, WaveBuffers wb,
    int bounce, int countSlot, int workSlot, BatchTables bt)
{
    uint32_t n      = wb.counters[bounce * kCounterStride + countSlot];
    TraceCounters c = { 0, 0 };
    bool overflow   = false;
    ShadowLoader rays{ wb.shTag, wb.shOrg, wb.shDir };
    if constexpr (kBatch)
        persistentTrace<true, kCount>(s, n, wb.counters + bounce * kCounterStride + workSlot,
            BatchShadowLoader{ rays, bt.pathReq, bt.req }, OcclusionWriter{ wb.shTag, wb.occluded },
            g_stack + threadIdx.x, kTraceBlock, c, overflow);
    else
        persistentTrace<true, kCount>(s, n, wb.counters + bounce * kCounterStride + workSlot, rays,
            OcclusionWriter{ wb.shTag, wb.occluded }, g_stack + threadIdx.x, kTraceBlock, c, overflow);
    if (kCount)
    {
        atomicAdd(statPtr(wb, 5), c.nodes);
        atomicAdd(statPtr(wb, 6), c.tris);
    }
    if (overflow)
        atomicAdd(statPtr(wb, 4), 1ull);
}

template <bool kCount, bool kBatch>
__global__ void __launch_bounds__(kTraceBlock, kTraceBlocksPerSM) k_trace_shadow_transparent(DevScene s,
    WaveBuffers wb, int bounce, BatchTables bt)
{
    uint32_t n      = wb.counters[bounce * kCounterStride + CNT_SHADOW];
    TraceCounters c = { 0, 0 };
    bool overflow   = false;
    TransparentShadowLoader rays{ ShadowLoader{ wb.shTag, wb.shOrg, wb.shDir }, wb.shadePoint };
    if constexpr (kBatch)
        persistentTrace<false, kCount>(s, n, wb.counters + bounce * kCounterStride + CNT_SHADOW_WORK,
            BatchTransparentShadowLoader{ rays, bt.pathReq, bt.req },
            TransparentShadowWriter{ wb.shTag, wb.shadePoint, wb.pendSlot }, g_stack + threadIdx.x,
            kTraceBlock, c, overflow);
    else
        persistentTrace<false, kCount>(s, n, wb.counters + bounce * kCounterStride + CNT_SHADOW_WORK, rays,
            TransparentShadowWriter{ wb.shTag, wb.shadePoint, wb.pendSlot }, g_stack + threadIdx.x,
            kTraceBlock, c, overflow);
    if (kCount)
    {
        atomicAdd(statPtr(wb, 5), c.nodes);
        atomicAdd(statPtr(wb, 6), c.tris);
    }
    if (overflow)
        atomicAdd(statPtr(wb, 4), 1ull);
}

// -------------------------------------------------------------------------------- shading
// ShadeFunctions.slang:51-89
AGB_DN v3 shadeDistantLight(const agb_distant_light& l, const Mat& m, const MatCommon& mc,
    const Frame& fr, v3 V, Rng& rng, v3& dirOut)
{
    v2 r    = random2D(rng);
    v3 L    = sampleCone(r, ld3(l.direction), l.cos_radius);
    v3 bsdf = evaluateMaterial(m, mc, fr, V, L);
    if (isBlack(bsdf))
    {
        dirOut = splat(0.f);
        return splat(0.f);
    }
    dirOut = L;
    return ld3(l.color_and_intensity) * l.color_and_intensity[3] * bsdf;
}

__device__ __forceinline__ void accumulateSegment(WaveBuffers& wb, uint32_t p, int bounce,
    uint32_t flags, uint32_t rayType, v3 direct, v3 indirect, float clampLum)
{
    if (bounce == 0)
    {
        wb.outDirect[p] = make_float4(direct.x, direct.y, direct.z, 0.f);
        float4 ind      = make_float4(indirect.x, indirect.y, indirect.z, 0.f);
        if (pfMisLobe(flags) == DIFFUSE_LOBE)
            wb.outDiffuse[p] = ind;
        else
            wb.outGlossy[p] = ind;
        return;
    }
    v3 radiance = direct + indirect;
    if (clampLum > 0.f)
    {
        float lum = luminance(radiance);
        if (lum > clampLum)
            radiance *= clampLum / lum;
        if (isnan(radiance.x) || isnan(radiance.y) || isnan(radiance.z) || isinf(radiance.x) ||
            isinf(radiance.y) || isinf(radiance.z))
            radiance = splat(0.f);
    }
    float4* dst = rayType == DIFFUSE_LOBE ? wb.outDiffuse + p : wb.outGlossy + p;
    float4 a    = *dst;
    *dst        = make_float4(a.x + radiance.x, a.y + radiance.y, a.z + radiance.z, 0.f);
}

// A shading point handed from k_shade to k_shade_scatter: kShadePointWords float4 per point,
// stored word-major (word k of point j at k * stride + j) so both kernels access it coalesced.
AGB_D void storeShadePoint(float4* sp, uint32_t stride, uint32_t j, const Mat& m, int32_t mi,
    uint32_t slots, uint32_t p, const MatCommon& c, const Frame& fr, v3 V, v3 pos, v3 geomPos)
{
    float4* w = sp + j;
    w[0 * size_t(stride)] = make_float4(m.baseColor.x, m.baseColor.y, m.baseColor.z, m.specularRoughness);
    w[1 * size_t(stride)] = make_float4(m.coatRoughness, __int_as_float(mi), __uint_as_float(slots),
        __uint_as_float(p));
    w[2 * size_t(stride)] = make_float4(c.mainRough.x, c.mainRough.y, c.mainTangent.x, c.mainTangent.y);
    w[3 * size_t(stride)] = make_float4(c.mainTangent.z, c.coatTangent.x, c.coatTangent.y, c.coatTangent.z);
    w[4 * size_t(stride)] = make_float4(c.diffuseColor.x, c.diffuseColor.y, c.diffuseColor.z,
        c.subsurfaceColor.x);
    w[5 * size_t(stride)] = make_float4(c.subsurfaceColor.y, c.subsurfaceColor.z, V.x, V.y);
    w[6 * size_t(stride)] = make_float4(V.z, fr.N.x, fr.N.y, fr.N.z);
    w[7 * size_t(stride)] = make_float4(fr.X.x, fr.X.y, fr.X.z, fr.Y.x);
    w[8 * size_t(stride)] = make_float4(fr.Y.y, fr.Y.z, pos.x, pos.y);
    w[9 * size_t(stride)] = make_float4(pos.z, geomPos.x, geomPos.y, geomPos.z);
}
AGB_D void loadShadePoint(const DevScene& s, const float4* sp, uint32_t stride, uint32_t j, Mat& m,
    uint32_t& slots, uint32_t& p, MatCommon& c, Frame& fr, v3& V, v3& pos, v3& geomPos)
{
    const float4* w = sp + j;
    float4 a = w[0], b = w[1 * size_t(stride)], q2 = w[2 * size_t(stride)], q3 = w[3 * size_t(stride)];
    float4 q4 = w[4 * size_t(stride)], q5 = w[5 * size_t(stride)], q6 = w[6 * size_t(stride)];
    float4 q7 = w[7 * size_t(stride)], q8 = w[8 * size_t(stride)], q9 = w[9 * size_t(stride)];
    m.b                 = s.materials + __float_as_int(b.y);
    m.baseColor         = v3{ a.x, a.y, a.z };
    m.specularRoughness = a.w;
    m.coatRoughness     = b.x;
    m.emissionColor     = splat(0.f); // applied by k_shade
    m.opacity           = splat(1.f); // applied by k_shade
    slots               = __float_as_uint(b.z);
    p                   = __float_as_uint(b.w);
    c.mainRough         = v2{ q2.x, q2.y };
    c.mainTangent       = v3{ q2.z, q2.w, q3.x };
    c.coatTangent       = v3{ q3.y, q3.z, q3.w };
    c.diffuseColor      = v3{ q4.x, q4.y, q4.z };
    c.subsurfaceColor   = v3{ q4.w, q5.x, q5.y };
    V                   = v3{ q5.z, q5.w, q6.x };
    fr.N                = v3{ q6.y, q6.z, q6.w };
    fr.X                = v3{ q7.x, q7.y, q7.z };
    fr.Y                = v3{ q7.w, q8.x, q8.y };
    pos                 = v3{ q8.z, q8.w, q9.x };
    geomPos             = v3{ q9.y, q9.z, q9.w };
}

// Per-path view of a wave's request: the whole wave's values for a single-request wave, the
// path's request's for a batched one.
struct PathRequest
{
    uint32_t local, pixels, samples, width, sampleBase, aovSample;
    int32_t traceDepth;
    float* aovDepth;
    float4* aovNormal;
    float4* aovAlbedo;
    float4* aovMotion;
};
template <bool kBatch>
AGB_D PathRequest pathRequest(const WaveParams& wp, const WaveBuffers& wb, const BatchTables& bt, uint32_t p,
    uint32_t& r, int depth)
{
    if constexpr (kBatch)
    {
        r                     = bt.pathReq[p];
        const BatchRequest& q = bt.req[r];
        return PathRequest{ p - q.pathOffset, q.pixels, q.samples, q.width, q.sampleBase, q.aovSample, q.traceDepth,
            q.aovDepth, q.aovNormal, q.aovAlbedo, q.aovMotion };
    }
    else
    {
        r = 0;
        return PathRequest{ p, wp.pixels, wp.samples, wp.width, wp.sampleBase, wp.aovSample, depth, wb.aovDepth,
            wb.aovNormal, wb.aovAlbedo, wb.aovMotion };
    }
}
AGB_D float bounceClamp(const agb_frame_data& f)
{
    return f.indirect_bounce_clamp_scale > 0.f ? f.max_luminance * f.indirect_bounce_clamp_scale : 0.f;
}

// kGraphs: the variant for scenes whose materials have node-graph programs (single-scene waves).
template <bool kBatch, bool kGraphs = false>
__global__ void __launch_bounds__(kShadeBlock, kShadeMinBlocks) k_shade(DevScene s, agb_frame_data f,
    WaveParams wp, WaveBuffers wb, int bounce, int cur, int depthLimit, BatchTables bt)
{
    uint32_t n      = wb.counters[bounce * kCounterStride + CNT_RAYS];
    uint32_t stride = gridDim.x * blockDim.x;
    // Warp-uniform loop: every lane of a warp runs the same number of iterations so the queue
    // appends at the end of the body are executed by the whole warp.
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride)
    {
        uint32_t i     = base + threadIdx.x;
        bool valid     = i < n;
        // A camera ray the ground plane turned into a reflection ray has nothing to shade here.
        if (valid && !depthLimit && s.ground.enabled && wb.hitInst[i] == kGroundAbsorbed)
            valid = false;
        bool pushNext  = false;
        uint32_t slots = 0;
        uint32_t p     = 0;
        v3 nextO = splat(0.f), nextD = splat(0.f);
        if (valid)
        {
            p          = wb.rayPath[cur][i];
            uint32_t r;
            const PathRequest q = pathRequest<kBatch>(wp, wb, bt, p, r, f.trace_depth);
            const agb_frame_data& F = kBatch ? bt.frames[r] : f;
            const DevScene& S       = kBatch ? bt.scenes[bt.req[r].scene] : s;
            const float clampLum    = bounceClamp(F);
            const v2 screen         = kBatch ? v2{ float(bt.req[r].width), float(bt.req[r].height) }
                                             : v2{ float(wp.width), float(wp.height) };
            float4 d4  = wb.rayDir[cur][i];
            v3 dir     = v3{ d4.x, d4.y, d4.z };
            uint32_t flags = wb.flags[p];
            float4 c4  = wb.contrib[p];
            v3 contrib = v3{ c4.x, c4.y, c4.z };
            uint32_t rayType = pfRayType(flags);
            bool primary = (flags & PF_PRIMARY) != 0;
            uint32_t pixel = pathPixel(q.local, q.pixels, q.samples);
            v2 pixel2 = v2{ float(pixel % q.width), float(pixel / q.width) };
            bool bg = primary || rayType == TRANSMISSION_LOBE || rayType == GROUND_PLANE_REFLECTION_RAY;
            // A batched request whose trace depth is this bounce takes the depth-limit segment here.
            if (depthLimit || (kBatch && bounce == q.traceDepth))
            {
                v3 direct = evaluateEnvironment(S, dir, bg, pixel2, screen) * contrib;
                float4 li = wb.lastIndirect[p];
                accumulateSegment(wb, p, bounce, flags, rayType, direct, v3{ li.x, li.y, li.z },
                    clampLum);
            }
            else
            {
                float4 h  = wb.hitTUV[i];
                int32_t inst = wb.hitInst[i];
                bool aov = primary && q.sampleBase + pathSample(q.local, q.pixels, q.samples) == q.aovSample;
                if (inst < 0)
                {
                    if (aov)
                    {
                        // Miss AOVs (MainEntryPoints.slang:380-406); the guide normal faces back
                        // along the ray.
                        q.aovDepth[pixel]  = F.sky_view_z;
                        q.aovNormal[pixel] = make_float4(-dir.x, -dir.y, -dir.z, 1.f);
                        q.aovAlbedo[pixel] = make_float4(0.f, 0.f, 0.f, 0.1f);
                        q.aovMotion[pixel] = skyMotion(F.camera_view_proj, F.camera_view_proj_prev,
                            dir, screen.x, screen.y);
                    }
                    v3 direct = bg ? evaluateEnvironment(S, dir, true, pixel2, screen) * contrib
                                   : splat(0.f);
                    accumulateSegment(wb, p, bounce, flags, rayType, direct, splat(0.f), clampLum);
                }
                else
                {
                    Rng rng;
                    {
                        uint2 r = wb.rng[p];
                        rng     = Rng{ r.x, r.y };
                    }
                    const DevInstance& in = S.instances[inst];
                    v3 V       = -dir;
                    Shading sh = computeShading(S, in, uint32_t(__float_as_int(h.w)), h.y, h.z);
                    v2 baseUV  = sh.uv;
                    bool hitLayer = false;
                    int32_t mi    = 0;
                    Mat m;
                    v3 matNormal = sh.N;
                    bool genNormal = false;
                    float P = 0.f;
                    for (int li = in.layerCount; li >= 0; li--)
                    {
                        mi = 0;
                        if (li == 0)
                        {
                            mi    = in.material;
                            sh.uv = baseUV;
                        }
                        else
                        {
                            const DevLayer& L = S.layers[in.layerOffset + li - 1];
                            mi = L.material;
                            v2 uv = v2{ 0.f, 0.f };
                            float b3[3] = { sh.bary.x, sh.bary.y, sh.bary.z };
                            for (int q = 0; q < 3; q++)
                            {
                                v2 t = v2{ __ldg(L.texcoords + 2 * size_t(sh.idx[q])),
                                    __ldg(L.texcoords + 2 * size_t(sh.idx[q]) + 1) };
                                uv = uv + t * b3[q];
                            }
                            sh.uv = uv;
                        }
                        matNormal = sh.N;
                        m = loadMaterial<kGraphs>(S, mi, sh, matNormal, genNormal, &in);
                        if (!primary && F.is_path_regularization_enabled)
                        {
                            float fl = lerpf(0.05f, lerpf(0.05f, 0.35f, F.path_regularization_strength),
                                saturatef(float(bounce) / 3.f));
                            m.specularRoughness = m.specularRoughness > fl ? m.specularRoughness : fl;
                            m.coatRoughness     = m.coatRoughness > fl ? m.coatRoughness : fl;
                        }
                        if (aov)
                        {
                            // Hit AOVs for every layer evaluated (HitShaderEntryPoints.slang:149-233).
                            float4 o4 = wb.rayOrg[cur][i];
                            v3 hw     = v3{ o4.x, o4.y, o4.z } + dir * h.x;
                            float vz  = viewDepth(F.camera_inv_view, hw);
                            v3 gn     = normalize(matNormal);
                            q.aovDepth[pixel]  = vz;
                            q.aovNormal[pixel] = make_float4(gn.x, gn.y, gn.z,
                                m.specularRoughness > 0.05f ? m.specularRoughness : 0.05f);
                            q.aovAlbedo[pixel] = make_float4(m.baseColor.x, m.baseColor.y,
                                m.baseColor.z, m.metalness());
                            q.aovMotion[pixel] = surfaceMotion(F.camera_view_proj,
                                F.camera_view_proj_prev, F.camera_inv_view_prev, hw, vz, screen.x,
                                screen.y);
                        }
                        v3 transparency = splat(1.f) - m.opacity;
                        P        = luminance(transparency);
                        hitLayer = random2D(rng).x >= P;
                        if (hitLayer)
                            break;
                        contrib *= transparency / P;
                    }
                    if (!hitLayer)
                    {
                        // No layer absorbed the ray: continue straight on (skipContribution).
                        nextO    = sh.geomPosition;
                        nextD    = dir;
                        pushNext = true;
                        wb.lastIndirect[p] = make_float4(0.f, 0.f, 0.f, 0.f);
                    }
                    else
                    {
                        Frame fr = Frame{ sh.N, sh.X, sh.Y };
                        if (genNormal)
                        {
                            fr.N = matNormal;
                            buildBasis(fr.N, fr.X, fr.Y);
                        }
                        // The Standard Surface values every BSDF call at this point shares
                        // (each reference call recomputes the same values).
                        const MatCommon mc = prepare(m, fr);
                        v3 emission = m.emissionColor * m.emission() * lerp3(splat(1.f), m.coatColor(), m.coat());
                        v3 so = dot(V, fr.N) < 0.f ? sh.geomPosition : sh.position;
                        float4* pslot = wb.pendSlot + size_t(p) * kMaxShadowSlots;
                        float4* pdir  = wb.shDir + size_t(p) * kMaxShadowSlots;
                        int nl = F.distant_light_count;
                        if (!F.is_denoising_aovs_enabled && nl > 1)
                        {
                            for (int l = 0; l < nl && l < 4; l++)
                            {
                                if (F.distant_lights[l].color_and_intensity[3] <= 0.f)
                                    continue;
                                v3 sd;
                                v3 r = shadeDistantLight(F.distant_lights[l], m, mc, fr, V, rng, sd);
                                if (isBlack(r))
                                    continue;
                                pslot[l] = make_float4(r.x, r.y, r.z, 0.f);
                                pdir[l]  = make_float4(sd.x, sd.y, sd.z, 0.f);
                                slots |= 1u << l;
                            }
                        }
                        else if (nl > 0)
                        {
                            float w[4];
                            float total = 0.f;
                            for (int l = 0; l < nl && l < 4; l++)
                            {
                                const float* ci = F.distant_lights[l].color_and_intensity;
                                w[l] = luminance(v3{ ci[0], ci[1], ci[2] }) * ci[3];
                                total += w[l];
                            }
                            int idx = 0;
                            float selPdf = 1.f / float(nl);
                            if (total > 0.f)
                            {
                                float r = random2D(rng).x * total;
                                float cum = 0.f;
                                for (int l = 0; l < nl && l < 4; l++)
                                {
                                    cum += w[l];
                                    if (r <= cum || l == nl - 1)
                                    {
                                        idx    = l;
                                        selPdf = w[l] / total;
                                        break;
                                    }
                                }
                            }
                            else
                                idx = int(random2D(rng).x * float(nl));
                            if (F.distant_lights[idx].color_and_intensity[3] > 0.f)
                            {
                                v3 sd;
                                v3 r = shadeDistantLight(F.distant_lights[idx], m, mc, fr, V, rng, sd);
                                r    = r / fmaxf_(selPdf, 1e-4f);
                                if (!isBlack(r))
                                {
                                    pslot[0] = make_float4(r.x, r.y, r.z, 0.f);
                                    pdir[0]  = make_float4(sd.x, sd.y, sd.z, 0.f);
                                    slots |= 1u;
                                }
                            }
                        }
                        contrib *= m.opacity / (1.f - P);
                        // Hand the shading point to k_shade_scatter (environment MIS, the next
                        // ray, Russian roulette), which runs with only those paths in its warps.
                        wb.pendEmission[p] = make_float4(emission.x, emission.y, emission.z, 0.f);
                        wb.shOrg[p]        = make_float4(so.x, so.y, so.z, 0.f);
                        uint32_t j = warpAppend(wb.counters + bounce * kCounterStride + CNT_SCATTER, true);
                        storeShadePoint(wb.shadePoint, wp.paths, j, m, mi, slots, p, mc, fr, V,
                            sh.position, sh.geomPosition);
                        slots = 0;
                    }
                    wb.rng[p]     = make_uint2(rng.x, rng.y);
                    wb.contrib[p] = make_float4(contrib.x, contrib.y, contrib.z, 0.f);
                    wb.flags[p]   = flags;
                }
            }
        }
        // Warp-aggregated append of the straight-through rays (all lanes of the warp reach this
        // point together).
        __syncwarp();
        uint32_t slotNext = warpAppend(wb.counters + (bounce + 1) * kCounterStride + CNT_RAYS, pushNext);
        if (pushNext)
        {
            wb.rayOrg[cur ^ 1][slotNext]  = make_float4(nextO.x, nextO.y, nextO.z, kRayTMin);
            wb.rayDir[cur ^ 1][slotNext]  = make_float4(nextD.x, nextD.y, nextD.z, __int_as_float(0x7f800000));
            wb.rayPath[cur ^ 1][slotNext] = p;
        }
    }
}

// The hit shading after k_shade, in two kernels over the compacted shading points, each holding
// one of the large Standard Surface entry points (the shading kernels' speed follows their
// instruction-cache footprint):
//   k_shade_scatter  draws the environment-MIS random pair and samples the BSDF with it
//                    (ShadeFunctions.slang:146-163), samples the indirect ray and applies Russian
//                    roulette (ShadeFunctions.slang:263-310, HitShaderEntryPoints.slang:362-486),
//                    appends the next ray and hands the MIS sample to k_shade_mis;
//   k_shade_mis      evaluates both halves of the environment MIS (ShadeFunctions.slang:135-259:
//                    environment lookup, environment sample, evaluateMaterialAndPDF with the same
//                    random pair), sets the pending-record bits and appends the resolve entry and
//                    the shadow rays.
// The random numbers are drawn in the reference's order (MIS pair, indirect pair, roulette); the
// MIS evaluation consumes none, so running it after the indirect sampling changes no value.

// MIS sample handed from k_shade_scatter to k_shade_mis: kMisWords float4 per shading point,
// word-major like the shading point.
AGB_D void storeMis(float4* mp, uint32_t stride, uint32_t j, v3 L, float pdf, v3 bsdf, int lobe, v2 rnd,
    uint32_t bitsBase)
{
    float4* w             = mp + j;
    w[0]                  = make_float4(L.x, L.y, L.z, pdf);
    w[1 * size_t(stride)] = make_float4(bsdf.x, bsdf.y, bsdf.z, __int_as_float(lobe));
    w[2 * size_t(stride)] = make_float4(rnd.x, rnd.y, __uint_as_float(bitsBase), 0.f);
}

template <bool kBatch>
__global__ void __launch_bounds__(kShadeBlock, kShadeMinBlocks) k_shade_scatter(DevScene s,
    agb_frame_data f, WaveParams wp, WaveBuffers wb, int bounce, int cur, BatchTables bt)
{
    uint32_t n      = wb.counters[bounce * kCounterStride + CNT_SCATTER];
    uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride)
    {
        uint32_t j     = base + threadIdx.x;
        bool valid     = j < n;
        bool pushNext  = false;
        uint32_t p     = 0;
        v3 nextO = splat(0.f), nextD = splat(0.f);
        if (valid)
        {
            Mat m;
            MatCommon mc;
            Frame fr;
            v3 V, shPosition, shGeomPosition;
            uint32_t slots;
            loadShadePoint(s, wb.shadePoint, wp.paths, j, m, slots, p, mc, fr, V, shPosition,
                shGeomPosition);
            const agb_frame_data& F = kBatch ? bt.frames[bt.pathReq[p]] : f;
            uint32_t flags = wb.flags[p];
            float4 c4      = wb.contrib[p];
            v3 contrib     = v3{ c4.x, c4.y, c4.z };
            uint32_t rayType = pfRayType(flags);
            Rng rng;
            {
                uint2 r = wb.rng[p];
                rng     = Rng{ r.x, r.y };
            }
            // Environment MIS, BSDF half's sample (one random pair for both halves).
            v2 rnd = random2D(rng);
            v3 Lmis;
            float mpdf;
            int misLobe;
            v3 bsdfMis = sampleMaterial(m, mc, fr, V, rnd, Lmis, mpdf, misLobe);
            bool alpha = (flags & PF_ALPHA) != 0;
            alpha = !(!alpha && rayType == TRANSMISSION_LOBE);
            flags = alpha ? (flags | PF_ALPHA) : (flags & ~PF_ALPHA);
            // setupIndirectLightRay (ShadeFunctions.slang:263-310)
            int nextType;
            v3 nextContrib = splat(1.f);
            {
                v3 L;
                float pdf;
                int lobe;
                v3 bsdf = sampleMaterial(m, mc, fr, V, random2D(rng), L, pdf, lobe);
                if (isBlack(bsdf))
                    nextType = NO_SECONDARY_RAY;
                else
                {
                    bool tr = lobe == TRANSMISSION_LOBE;
                    nextO = (dot(V, fr.N) < 0.f || tr) ? shGeomPosition : shPosition;
                    nextD = L;
                    nextContrib = bsdf / pdf;
                    nextType = lobe;
                }
            }
            bool ended = nextType == NO_SECONDARY_RAY;
            // Pending-record bits that do not depend on the MIS result.
            uint32_t bitsBase = slots;
            if (bounce == 0)
                bitsBase |= RS_DEPTH0;
            else if (rayType == DIFFUSE_LOBE)
                bitsBase |= RS_DIFFUSE_ROUTE;
            storeMis(wb.misPoint, wp.paths, j, Lmis, mpdf, bsdfMis, misLobe, rnd, bitsBase);
            wb.pendSegContrib[p] = make_float4(contrib.x, contrib.y, contrib.z, 0.f);
            flags &= ~PF_PRIMARY;
            if (nextType == TRANSMISSION_LOBE)
                flags ^= PF_INSIDE;
            contrib *= nextContrib;
            if (F.is_russian_roulette_enabled && bounce + 1 >= F.russian_roulette_start_depth)
            {
                float mx   = fmaxf_(contrib.x, fmaxf_(contrib.y, contrib.z));
                float surv = clampf(mx, 0.05f, 1.f);
                if (random2D(rng).x > surv)
                    ended = true;
                else
                    contrib = contrib / surv;
            }
            flags    = pfSetRayType(flags, uint32_t(nextType));
            pushNext = !ended;
            wb.rng[p]     = make_uint2(rng.x, rng.y);
            wb.contrib[p] = make_float4(contrib.x, contrib.y, contrib.z, 0.f);
            wb.flags[p]   = flags;
        }
        // Warp-aggregated append of the next rays (all lanes of the warp reach this point together).
        __syncwarp();
        uint32_t slotNext = warpAppend(wb.counters + (bounce + 1) * kCounterStride + CNT_RAYS, pushNext);
        if (pushNext)
        {
            wb.rayOrg[cur ^ 1][slotNext]  = make_float4(nextO.x, nextO.y, nextO.z, kRayTMin);
            wb.rayDir[cur ^ 1][slotNext]  = make_float4(nextD.x, nextD.y, nextD.z, __int_as_float(0x7f800000));
            wb.rayPath[cur ^ 1][slotNext] = p;
        }
    }
}

template <bool kBatch>
__global__ void __launch_bounds__(kShadeBlock, kShadeMinBlocks) k_shade_mis(DevScene s,
    agb_frame_data f, WaveParams wp, WaveBuffers wb, int bounce, BatchTables bt)
{
    uint32_t n      = wb.counters[bounce * kCounterStride + CNT_SCATTER];
    uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride)
    {
        uint32_t j     = base + threadIdx.x;
        bool valid     = j < n;
        uint32_t slots = 0;
        uint32_t p     = 0;
        if (valid)
        {
            Mat m;
            MatCommon mc;
            Frame fr;
            v3 V, shPosition, shGeomPosition;
            loadShadePoint(s, wb.shadePoint, wp.paths, j, m, slots, p, mc, fr, V, shPosition,
                shGeomPosition);
            const float4* w = wb.misPoint + j;
            float4 w0 = w[0], w1 = w[1 * size_t(wp.paths)], w2 = w[2 * size_t(wp.paths)];
            v3 L          = v3{ w0.x, w0.y, w0.z };
            float mpdf    = w0.w;
            v3 bsdf       = v3{ w1.x, w1.y, w1.z };
            int misLobe   = __float_as_int(w1.w);
            v2 rnd        = v2{ w2.x, w2.y };
            uint32_t bits = __float_as_uint(w2.z);
            uint32_t r;
            const PathRequest q = pathRequest<kBatch>(wp, wb, bt, p, r, f.trace_depth);
            const DevScene& S   = kBatch ? bt.scenes[bt.req[r].scene] : s;
            const v2 screen     = kBatch ? v2{ float(bt.req[r].width), float(bt.req[r].height) }
                                         : v2{ float(wp.width), float(wp.height) };
            uint32_t pixel = pathPixel(q.local, q.pixels, q.samples);
            v2 pixel2      = v2{ float(pixel % q.width), float(pixel / q.width) };
            float4* pslot  = wb.pendSlot + size_t(p) * kMaxShadowSlots;
            float4* pdir   = wb.shDir + size_t(p) * kMaxShadowSlots;
            // Environment MIS (ShadeFunctions.slang:135-259).
            bool mis = false;
            if (misLobe != TRANSMISSION_LOBE)
            {
                v3 lr = evaluateEnvironment(S, L, false, pixel2, screen);
                if (!isBlack(lr) && !isBlack(bsdf))
                {
                    float lpdf = S.env.has_light_tex && S.envLight.data
                        ? luminance(lr) / S.env.light_tex_luminance_integral
                        : divPi(0.25f);
                    v3 res = lr * misWeight(mpdf, lpdf) * bsdf / mpdf;
                    pslot[4] = make_float4(res.x, res.y, res.z, 0.f);
                    pdir[4]  = make_float4(L.x, L.y, L.z, 0.f);
                    slots |= 1u << 4;
                }
                float lpdf;
                lr = sampleEnvironment(S, rnd, L, lpdf);
                int el;
                bsdf = evaluateMaterialAndPDF(m, mc, fr, V, L, rnd, mpdf, el);
                if (!isBlack(lr) && !isBlack(bsdf))
                {
                    v3 res = lr * misWeight(lpdf, mpdf) * bsdf / lpdf;
                    pslot[5] = make_float4(res.x, res.y, res.z, 0.f);
                    pdir[5]  = make_float4(L.x, L.y, L.z, 0.f);
                    slots |= 1u << 5;
                }
                mis = (slots & 0x30u) != 0;
            }
            bits |= slots;
            if (mis)
            {
                bits |= RS_MIS;
                wb.flags[p] = pfSetMisLobe(wb.flags[p], uint32_t(misLobe));
            }
            if (bounce == 0 && pfMisLobe(wb.flags[p]) == DIFFUSE_LOBE)
                bits |= RS_DIFFUSE_ROUTE;
            wb.pendBits[p] = bits;
            wb.occluded[p] = 0u;
        }
        // Warp-aggregated appends (all lanes of the warp reach this point together).
        __syncwarp();
        uint32_t slotRes = warpAppend(wb.counters + bounce * kCounterStride + CNT_RESOLVE, valid);
        if (valid)
            wb.resolveList[slotRes] = p;
        // Shadow rays: variable count per lane, warp prefix sum then one atomic.
        uint32_t cnt = __popc(slots);
        uint32_t incl = cnt;
        int lane = threadIdx.x & 31;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1)
        {
            uint32_t v = __shfl_up_sync(0xffffffffu, incl, off);
            if (lane >= off)
                incl += v;
        }
        uint32_t total = __shfl_sync(0xffffffffu, incl, 31);
        uint32_t sbase = 0;
        if (lane == 31 && total)
            sbase = atomicAdd(wb.counters + bounce * kCounterStride + CNT_SHADOW, total);
        sbase = __shfl_sync(0xffffffffu, sbase, 31);
        uint32_t wpos = sbase + incl - cnt;
        for (uint32_t k = 0; k < uint32_t(kMaxShadowSlots); k++)
            if (slots & (1u << k))
                wb.shTag[wpos++] = (p << 3) | k;
    }
}

// Applies shadow visibility to the pending contributions and accumulates the segment.
template <bool kBatch>
__global__ void k_resolve(agb_frame_data f, WaveBuffers wb, int bounce, BatchTables bt)
{
    uint32_t n      = wb.counters[bounce * kCounterStride + CNT_RESOLVE];
    uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    {
        uint32_t p    = wb.resolveList[i];
        const float clampLum = bounceClamp(kBatch ? bt.frames[bt.pathReq[p]] : f);
        uint32_t bits = wb.pendBits[p];
        uint32_t occ  = wb.occluded[p];
        float4 e      = wb.pendEmission[p];
        v3 direct     = v3{ e.x, e.y, e.z };
        const float4* ps = wb.pendSlot + size_t(p) * kMaxShadowSlots;
        for (int k = 0; k < 4; k++)
            if (bits & (1u << k))
            {
                float vis = (occ >> k) & 1u ? 0.f : 1.f;
                float4 c  = ps[k];
                direct += splat(vis) * v3{ c.x, c.y, c.z };
            }
        v3 indirect = splat(0.f);
        if (bits & RS_MIS)
        {
            v3 misr = splat(0.f);
            for (int k = 4; k < 6; k++)
                if (bits & (1u << k))
                {
                    float vis = (occ >> k) & 1u ? 0.f : 1.f;
                    float4 c  = ps[k];
                    misr += splat(vis) * v3{ c.x, c.y, c.z };
                }
            indirect = misr;
        }
        float4 sc4 = wb.pendSegContrib[p];
        v3 sc      = v3{ sc4.x, sc4.y, sc4.z };
        direct *= sc;
        indirect *= sc;
        wb.lastIndirect[p] = make_float4(indirect.x, indirect.y, indirect.z, 0.f);
        if (bits & RS_DEPTH0)
        {
            wb.outDirect[p] = make_float4(direct.x, direct.y, direct.z, 0.f);
            float4 ind      = make_float4(indirect.x, indirect.y, indirect.z, 0.f);
            if (bits & RS_DIFFUSE_ROUTE)
                wb.outDiffuse[p] = ind;
            else
                wb.outGlossy[p] = ind;
            continue;
        }
        v3 radiance = direct + indirect;
        if (clampLum > 0.f)
        {
            float lum = luminance(radiance);
            if (lum > clampLum)
                radiance *= clampLum / lum;
            if (isnan(radiance.x) || isnan(radiance.y) || isnan(radiance.z) || isinf(radiance.x) ||
                isinf(radiance.y) || isinf(radiance.z))
                radiance = splat(0.f);
        }
        float4* dst = (bits & RS_DIFFUSE_ROUTE) ? wb.outDiffuse + p : wb.outGlossy + p;
        float4 a    = *dst;
        *dst        = make_float4(a.x + radiance.x, a.y + radiance.y, a.z + radiance.z, 0.f);
    }
}

// PathTracingCommon.slang:59-82
__device__ __forceinline__ void adjustRadiance(float maxLum, bool displayErrors, v3& r)
{
    float lum = luminance(r);
    if (lum > maxLum)
        r *= maxLum / lum;
    if (isnan(r.x) || isnan(r.y) || isnan(r.z))
        r = displayErrors ? v3{ __int_as_float(0x7f800000), 0.f, 0.f } : splat(0.f);
    else if (isinf(r.x) || isinf(r.y) || isinf(r.z))
        r = displayErrors ? v3{ 0.f, __int_as_float(0x7f800000), 0.f } : splat(0.f);
}

// ---------------------------------------------------------------------------- ground plane
// sampleGGXSmithBRDF (BSDFCommon.slang:331-366) with anisotropy 0, tangent space: a GGX-Smith
// VNDF half-vector (flipped for a lower-hemisphere view), the reflected direction and its PDF,
// and the microfacet BRDF D G2 F / (4 |V.z| |L.z|) with Schlick Fresnel (BSDFCommon.slang:115-118,
// 231-240, 310-327); black when V and L are in different hemispheres.
AGB_D v3 sampleGGXSmithBRDF(v3 V, v3 f0, float roughness, v2 r, v3& L, float& pdf)
{
    float a   = fmaxf_(0.0001f, sqr(roughness)); // roughnessToAlpha, MIN_ALPHA
    v2 alpha  = v2{ a, a };
    bool flip = V.z <= 0.f;
    v3 H      = sampleGGXVNDF(flip ? -V : V, alpha, r);
    H         = flip ? -H : H;
    L         = reflect(-V, H);
    pdf       = ggxVNDF(V, H, alpha) / (4.f * dot(V, H));
    if (!(V.z * L.z > 0.f))
        return splat(0.f);
    v3 Hn    = normalize(V + L);
    float D  = ggxNDF(Hn, alpha);
    float G2 = (dot(V, Hn) <= 0.f || dot(L, Hn) < 0.f)
        ? 0.f
        : 1.f / (1.f + ggxLambda(V, alpha) + ggxLambda(L, alpha));
    float w  = agb_fm::pow(1.f - dot(V, Hn), 5.f);
    v3 F     = f0 + (splat(1.f) - f0) * w;
    return F * (D * G2) / (4.f * fabsf(V.z) * fabsf(L.z));
}

// The ground plane for the primary rays of a bounce (evaluateGroundPlane, GroundPlane.slang:236-289,
// called first by the closest-hit and miss shaders while the ray is primary: the camera rays and
// the rays that passed through a transparent surface since, which stay primary), after their
// closest-hit traversal and before shading.  A ray that meets the plane from its front side
// nearer than its hit (any distance on a miss) draws from its own random stream, in the
// reference's order:
//   - with probability 1 - luminance(1 - reflection opacity) it becomes a matte reflection ray
//     (setupMatteReflectionIndirectLightRay): GGX-Smith sample about the plane's frame, the
//     contribution scaled by bsdf cos / pdf x opacity / (1 - Pr), the guide AOVs of the plane
//     written, the next segment appended as GROUND_PLANE_REFLECTION_RAY and the hit marked
//     absorbed.  A black BSDF sample leaves the ray unabsorbed with only the opacity scale;
//   - otherwise the contribution is scaled by the transparency / Pr and, with a shadow opacity,
//     an environment sample above the plane is traced as an opaque shadow ray (shadeMatteShadow,
//     GroundPlane.slang:71-104; counter CNT_GROUND_SHADOW of the bounce) whose colour factor
//     waits in the path's first pending slot until k_ground_shadow applies it.
__global__ void k_ground(DevScene s, agb_frame_data f, WaveParams wp, WaveBuffers wb, int bounce, int cur)
{
    const DevGroundPlane& g = s.ground;
    uint32_t n      = wb.counters[bounce * kCounterStride + CNT_RAYS];
    uint32_t stride = gridDim.x * blockDim.x;
    const v3 N = ld3(g.normal), X = ld3(g.tangent), Y = ld3(g.bitangent), P0 = ld3(g.position);
    v2 screen  = v2{ float(wp.width), float(wp.height) };
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += stride)
    {
        uint32_t i      = base + threadIdx.x;
        uint32_t p      = 0;
        bool reflectRay = false, shadowRay = false;
        v3 hitPos = splat(0.f), nextD = splat(0.f), shadowL = splat(0.f);
        if (i < n)
        {
            p         = wb.rayPath[cur][i];
            float4 o4 = wb.rayOrg[cur][i], d4 = wb.rayDir[cur][i];
            v3 o      = v3{ o4.x, o4.y, o4.z }, d = v3{ d4.x, d4.y, d4.z };
            // RayTCurrent(): the hit distance, or the ray's TMax (infinity) on a miss.
            float tCur = wb.hitInst[i] >= 0 ? wb.hitTUV[i].x : d4.w;
            // intersectGroundPlane (GroundPlane.slang:106-131).
            float planeDot = dot(d, N);
            bool onPlane   = false;
            float dist     = 0.f;
            if (!(planeDot >= 0.f))
            {
                dist    = dot(P0 - o, N) / planeDot;
                onPlane = !(dist < 0.f);
            }
            if ((wb.flags[p] & PF_PRIMARY) && onPlane && dist < tCur)
            {
                hitPos = o + d * dist;
                Rng rng;
                {
                    uint2 r = wb.rng[p];
                    rng     = Rng{ r.x, r.y };
                }
                // setupGroundPlaneRay (GroundPlane.slang:136-193).
                v3 color     = splat(1.f);
                bool decided = false;
                if (g.reflectionOpacity > 0.f)
                {
                    v3 transparency = splat(1.f - g.reflectionOpacity);
                    float Pr        = luminance(transparency);
                    if (random2D(rng).x >= Pr)
                    {
                        v3 V = v3{ dot(-d, X), dot(-d, Y), dot(-d, N) };
                        v3 L;
                        float pdf;
                        v2 r      = random2D(rng);
                        v3 bsdf   = sampleGGXSmithBRDF(V, ld3(g.reflectionColor), g.reflectionRoughness, r, L, pdf);
                        bsdf      = bsdf * fabsf(L.z);
                        if (!isBlack(bsdf))
                        {
                            nextD      = X * L.x + Y * L.y + N * L.z;
                            color      = bsdf / pdf;
                            reflectRay = true;
                        }
                        color   = color * (g.reflectionOpacity / (1.f - Pr));
                        decided = true;
                    }
                    else
                        color = transparency / Pr;
                }
                if (!decided && g.shadowOpacity > 0.f)
                {
                    v3 L;
                    float pdf;
                    sampleEnvironment(s, random2D(rng), L, pdf);
                    // Below the plane the light casts no shadow: the shadow blend is zero and the
                    // colour stays as it is.
                    if (!(dot(L, N) < 0.f))
                    {
                        shadowRay = true;
                        shadowL   = L;
                    }
                }
                wb.rng[p] = make_uint2(rng.x, rng.y);
                if (shadowRay)
                    wb.pendSlot[size_t(p) * kMaxShadowSlots] = make_float4(color.x, color.y, color.z, 0.f);
                else
                {
                    float4 c4     = wb.contrib[p];
                    wb.contrib[p] = make_float4(c4.x * color.x, c4.y * color.y, c4.z * color.z, 0.f);
                }
                if (reflectRay)
                {
                    wb.hitInst[i] = kGroundAbsorbed;
                    wb.flags[p]   = pfSetRayType(wb.flags[p] & ~PF_PRIMARY, GROUND_PLANE_REFLECTION_RAY);
                    if (wp.sampleBase + pathSample(p, wp.pixels, wp.samples) == wp.aovSample)
                    {
                        // writeGroundPlaneGuideAOVs (GroundPlane.slang:197-233).
                        uint32_t pixel      = pathPixel(p, wp.pixels, wp.samples);
                        float vz            = viewDepth(f.camera_inv_view, hitPos);
                        wb.aovDepth[pixel]  = vz;
                        wb.aovNormal[pixel] = make_float4(N.x, N.y, N.z, fmaxf_(g.reflectionRoughness, 0.05f));
                        wb.aovAlbedo[pixel] = make_float4(g.reflectionColor[0], g.reflectionColor[1],
                            g.reflectionColor[2], 0.f);
                        wb.aovMotion[pixel] = surfaceMotion(f.camera_view_proj, f.camera_view_proj_prev,
                            f.camera_inv_view_prev, hitPos, vz, screen.x, screen.y);
                    }
                }
            }
        }
        uint32_t slotNext = warpAppend(wb.counters + (bounce + 1) * kCounterStride + CNT_RAYS, reflectRay);
        if (reflectRay)
        {
            wb.rayOrg[cur ^ 1][slotNext]  = make_float4(hitPos.x, hitPos.y, hitPos.z, kRayTMin);
            wb.rayDir[cur ^ 1][slotNext]  = make_float4(nextD.x, nextD.y, nextD.z, __int_as_float(0x7f800000));
            wb.rayPath[cur ^ 1][slotNext] = p;
        }
        uint32_t slotShadow = warpAppend(wb.counters + bounce * kCounterStride + CNT_GROUND_SHADOW, shadowRay);
        if (shadowRay)
        {
            wb.shOrg[p]                           = make_float4(hitPos.x, hitPos.y, hitPos.z, 0.f);
            wb.shDir[size_t(p) * kMaxShadowSlots] = make_float4(shadowL.x, shadowL.y, shadowL.z, 0.f);
            wb.shTag[slotShadow]                  = p << 3;
            wb.occluded[p]                        = 0u;
        }
    }
}

// The matte shadow of the ground plane (GroundPlane.slang:171-182): the waiting colour factor is
// scaled by lerp(1, shadow colour, luminance(1 - 0) x shadow opacity) when the opaque shadow ray
// was blocked (by lerp(1, shadow colour, 0) = 1 otherwise), then multiplies the contribution, in
// the reference's order (contribution x (colour x blend)).
__global__ void k_ground_shadow(DevScene s, WaveBuffers wb, int bounce)
{
    const DevGroundPlane& g = s.ground;
    uint32_t n      = wb.counters[bounce * kCounterStride + CNT_GROUND_SHADOW];
    uint32_t stride = gridDim.x * blockDim.x;
    v3 blend = lerp3(splat(1.f), ld3(g.shadowColor), luminance(splat(1.f) - splat(0.f)) * g.shadowOpacity);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    {
        uint32_t p = wb.shTag[i] >> 3;
        float4 f4  = wb.pendSlot[size_t(p) * kMaxShadowSlots];
        v3 color   = v3{ f4.x, f4.y, f4.z };
        if (wb.occluded[p] & 1u)
            color = color * blend;
        float4 c4     = wb.contrib[p];
        wb.contrib[p] = make_float4(c4.x * color.x, c4.y * color.y, c4.z * color.z, 0.f);
    }
}

// The per-pixel accumulation of k_finalize: begin() reads the pixel's accumulation state, add()
// takes the wave's samples in sample order, end() writes the state back.
struct PixelAccum
{
    float4 mean, sum, comp, res;
    float2 mom;
    AGB_D void begin(const WaveParams& wp, const WaveBuffers& wb, uint32_t pixel)
    {
        mean = sum = comp = make_float4(0.f, 0.f, 0.f, 0.f);
        if ((wp.accumMode & AGB_ACCUM_RUNNING_MEAN) && wp.sampleBase > 0)
            mean = wb.accumMean[pixel];
        if ((wp.accumMode & AGB_ACCUM_KAHAN) && wp.sampleBase > 0)
        {
            sum  = wb.accumSum[pixel];
            comp = wb.accumComp[pixel];
        }
        res = mean;
        mom = make_float2(0.f, 0.f);
        if ((wp.accumMode & AGB_ACCUM_MOMENTS) && wp.sampleBase > 0)
            mom = wb.accumMoments[pixel];
    }
    // r: the sample's final radiance (rgb) and alpha; s: its sample index.
    AGB_D void add(const WaveParams& wp, float4 r, uint32_t s)
    {
        res = r;
        if (wp.accumMode & AGB_ACCUM_MOMENTS)
        {
            float l = luminance(v3{ r.x, r.y, r.z });
            mom     = make_float2(mom.x + l, mom.y + l * l);
        }
        if (wp.accumMode & AGB_ACCUM_RUNNING_MEAN)
        {
            if (s == 0)
                mean = res;
            else
            {
                float t  = __fdiv_rn(1.f, float(s + 1));
                float om = __fsub_rn(1.f, t);
                mean = make_float4(__fadd_rn(__fmul_rn(mean.x, om), __fmul_rn(res.x, t)),
                    __fadd_rn(__fmul_rn(mean.y, om), __fmul_rn(res.y, t)),
                    __fadd_rn(__fmul_rn(mean.z, om), __fmul_rn(res.z, t)),
                    __fadd_rn(__fmul_rn(mean.w, om), __fmul_rn(res.w, t)));
            }
        }
        if (wp.accumMode & AGB_ACCUM_KAHAN)
        {
            // Kahan-compensated sum: y = x - c; t = sum + y; c = (t - sum) - y; sum = t.
            float* sp = &sum.x;
            float* cp = &comp.x;
            const float* xp = &res.x;
#pragma unroll
            for (int q = 0; q < 4; q++)
            {
                float y  = __fsub_rn(xp[q], cp[q]);
                float tt = __fadd_rn(sp[q], y);
                cp[q]    = __fsub_rn(__fsub_rn(tt, sp[q]), y);
                sp[q]    = tt;
            }
        }
    }
    AGB_D void end(const WaveParams& wp, const WaveBuffers& wb, uint32_t pixel) const
    {
        if (wp.accumMode & AGB_ACCUM_MOMENTS)
            wb.accumMoments[pixel] = mom;
        if (wp.accumMode & AGB_ACCUM_RUNNING_MEAN)
            wb.accumMean[pixel] = mean;
        if (wp.accumMode & AGB_ACCUM_KAHAN)
        {
            wb.accumSum[pixel]  = sum;
            wb.accumComp[pixel] = comp;
        }
        if (wb.lastSample)
            wb.lastSample[pixel] = res;
    }
};

// The final radiance of path p (adjustRadiance of its direct + diffuse + glossy sum) and its alpha.
AGB_D float4 finalRadiance(const agb_frame_data& f, const WaveBuffers& wb, uint32_t p)
{
    float4 a = wb.outDirect[p], b = wb.outDiffuse[p], c = wb.outGlossy[p];
    v3 fin = (v3{ a.x, a.y, a.z } + v3{ b.x, b.y, b.z }) + v3{ c.x, c.y, c.z };
    adjustRadiance(f.max_luminance, f.is_display_errors_enabled != 0, fin);
    return make_float4(fin.x, fin.y, fin.z, (wb.flags[p] & PF_ALPHA) ? 1.f : 0.f);
}

// One pixel of k_finalize: the final radiance of each of the wave's samples in sample order, then
// the accumulation (paths of the pixel at pathBase + pathOf(pixel, k)).
AGB_D void finalizePixelImpl(const agb_frame_data& f, const WaveParams& wp, const WaveBuffers& wb, uint32_t pixel,
    uint32_t pathBase)
{
    PixelAccum acc;
    acc.begin(wp, wb, pixel);
    for (uint32_t k = 0; k < wp.samples; k++)
        acc.add(wp, finalRadiance(f, wb, pathBase + pathOf(pixel, k, wp.pixels, wp.samples)), wp.sampleBase + k);
    acc.end(wp, wb, pixel);
}

#if AGB_SAMPLE_INNER
// Single-scene waves with a pixel's samples side by side: the paths of a block's 256 pixels are
// one contiguous range, read in chunks of kFinalChunk samples per pixel by consecutive threads
// (whole 128-byte lines) into shared memory, from which each thread accumulates its pixel.
constexpr int kFinalChunk = 8;
__global__ void __launch_bounds__(256) k_finalize_staged(agb_frame_data f, WaveParams wp, WaveBuffers wb)
{
    __shared__ float4 stage[256 * (kFinalChunk + 1)];
    const uint32_t S = wp.samples;
    for (uint32_t pix0 = blockIdx.x * 256u; pix0 < wp.pixels; pix0 += gridDim.x * 256u)
    {
        const uint32_t npix  = min(256u, wp.pixels - pix0);
        const uint32_t pixel = pix0 + threadIdx.x;
        const bool valid     = threadIdx.x < npix;
        PixelAccum acc;
        if (valid)
            acc.begin(wp, wb, pixel);
        for (uint32_t k0 = 0; k0 < S; k0 += kFinalChunk)
        {
            const uint32_t kc = min(uint32_t(kFinalChunk), S - k0);
            __syncthreads();
            for (uint32_t e = threadIdx.x; e < npix * kc; e += 256)
            {
                const uint32_t j = e / kc, kk = e - j * kc;
                stage[j * (kFinalChunk + 1) + kk] = finalRadiance(f, wb, (pix0 + j) * S + k0 + kk);
            }
            __syncthreads();
            if (valid)
                for (uint32_t kk = 0; kk < kc; kk++)
                    acc.add(wp, stage[threadIdx.x * (kFinalChunk + 1) + kk], wp.sampleBase + k0 + kk);
        }
        if (valid)
            acc.end(wp, wb, pixel);
    }
}
#endif

template <bool kBatch>
__global__ void k_finalize(agb_frame_data f, WaveParams wp, WaveBuffers wbIn, BatchTables bt)
{
    uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t total = kBatch ? bt.pixelsTotal : wp.pixels;
    for (uint32_t gq = blockIdx.x * blockDim.x + threadIdx.x; gq < total; gq += stride)
    {
        // A batched wave finalizes every request's pixels: the request's accumulation targets,
        // sample range and frame.
        WaveParams wp2  = wp;
        WaveBuffers wb  = wbIn;
        uint32_t pixel  = gq;
        uint32_t pathBase = 0;
        uint32_t r = 0;
        if constexpr (kBatch)
        {
            r                     = batchRequestOfPixel(bt, gq);
            const BatchRequest& q = bt.req[r];
            pixel           = gq - q.pixelOffset;
            pathBase        = q.pathOffset;
            wp2.pixels      = q.pixels;
            wp2.sampleBase  = q.sampleBase;
            wp2.samples     = q.samples;
            wp2.accumMode   = q.accumMode;
            wb.accumMean    = q.accumMean;
            wb.accumSum     = q.accumSum;
            wb.accumComp    = q.accumComp;
            wb.lastSample   = q.lastSample;
            wb.accumMoments = q.accumMoments;
        }
        const agb_frame_data& F = kBatch ? bt.frames[r] : f;
        finalizePixelImpl(F, wp2, wb, pixel, pathBase);
    }
}


// ----------------------------------------------------------------------------- ray binning
// Between bounces the next rays are regrouped (a counting sort into kRayBins bins) so that the
// lanes of a traversal warp start from nearby points in similar directions and walk overlapping
// node sets: the origin's cell of a 16^3 grid over the scene bounds (Morton order) under the
// direction's octant.  A ray's result does not depend on its queue position, so images are
// unchanged.
AGB_D uint32_t rayBin(const WaveParams& wp, float4 o, float4 d)
{
    const float p[3] = { o.x, o.y, o.z };
    uint32_t c[3];
#pragma unroll
    for (int k = 0; k < 3; k++)
    {
        float t = (p[k] - wp.binLo[k]) * wp.binScale[k];
        int q   = t > 0.f ? int(t) : 0;
        c[k]    = uint32_t(q < 15 ? q : 15);
    }
    uint32_t m = 0;
#pragma unroll
    for (int b = 0; b < 4; b++)
        m |= (((c[0] >> b) & 1u) << (3 * b)) | (((c[1] >> b) & 1u) << (3 * b + 1)) |
            (((c[2] >> b) & 1u) << (3 * b + 2));
    uint32_t oct = (d.x < 0.f ? 1u : 0u) | (d.y < 0.f ? 2u : 0u) | (d.z < 0.f ? 4u : 0u);
    return (oct << 12) | m;
}

__global__ void k_bin_count(WaveParams wp, WaveBuffers wb, int bounce, int src)
{
    const uint32_t n    = wb.counters[bounce * kCounterStride + CNT_RAYS];
    const uint32_t step = gridDim.x * blockDim.x;
    const int lane      = threadIdx.x & 31;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += step)
    {
        const uint32_t i = base + threadIdx.x;
        const bool valid = i < n;
        const unsigned act = __ballot_sync(0xffffffffu, valid);
        if (valid)
        {
            uint32_t bin   = rayBin(wp, wb.rayOrg[src][i], wb.rayDir[src][i]);
            unsigned peers = __match_any_sync(act, bin);
            if (lane == __ffs(peers) - 1)
                atomicAdd(wb.binCount + bin, uint32_t(__popc(peers)));
        }
    }
}

// Exclusive prefix sums of the bin counts into the offsets (one block of 1024 threads, 32 bins
// each); the counts are cleared for the next use.
__global__ void __launch_bounds__(1024) k_bin_scan(WaveBuffers wb)
{
    __shared__ uint32_t part[1024];
    constexpr uint32_t per = kRayBins / 1024;
    const uint32_t t       = threadIdx.x;
    uint32_t local[per];
    uint32_t sum = 0;
#pragma unroll
    for (uint32_t k = 0; k < per; k++)
    {
        local[k] = wb.binCount[t * per + k];
        wb.binCount[t * per + k] = 0;
        sum += local[k];
    }
    part[t] = sum;
    __syncthreads();
    for (uint32_t off = 1; off < 1024; off <<= 1)
    {
        uint32_t v = t >= off ? part[t - off] : 0u;
        __syncthreads();
        part[t] += v;
        __syncthreads();
    }
    uint32_t run = part[t] - sum;
#pragma unroll
    for (uint32_t k = 0; k < per; k++)
    {
        wb.binOffset[t * per + k] = run;
        run += local[k];
    }
}

// Moves the rays of queue src into queue src ^ 1 in bin order.
__global__ void k_bin_scatter(WaveParams wp, WaveBuffers wb, int bounce, int src)
{
    const uint32_t n    = wb.counters[bounce * kCounterStride + CNT_RAYS];
    const uint32_t step = gridDim.x * blockDim.x;
    const int lane      = threadIdx.x & 31;
    const int dst       = src ^ 1;
    for (uint32_t base = blockIdx.x * blockDim.x; base < n; base += step)
    {
        const uint32_t i = base + threadIdx.x;
        const bool valid = i < n;
        const unsigned act = __ballot_sync(0xffffffffu, valid);
        if (valid)
        {
            float4 o       = wb.rayOrg[src][i];
            float4 d       = wb.rayDir[src][i];
            uint32_t path  = wb.rayPath[src][i];
            uint32_t bin   = rayBin(wp, o, d);
            unsigned peers = __match_any_sync(act, bin);
            int leader     = __ffs(peers) - 1;
            uint32_t pos   = 0;
            if (lane == leader)
                pos = atomicAdd(wb.binOffset + bin, uint32_t(__popc(peers)));
            pos = __shfl_sync(peers, pos, leader) + uint32_t(__popc(peers & ((1u << lane) - 1u)));
            wb.rayOrg[dst][pos]  = o;
            wb.rayDir[dst][pos]  = d;
            wb.rayPath[dst][pos] = path;
        }
    }
}

// ------------------------------------------------------------------------------ launchers
// One wave: `depth` bounces (the frame's trace depth; a batched wave's deepest request), the
// ground plane's kernels when the scene has one (single-request waves only), transparent or
// opaque shadows as `forceOpaque` says.
template <bool kBatch>
void launchWaveT(const DevScene& s, const agb_frame_data& f, const WaveParams& wp, const WaveBuffers& wb,
    const BatchTables& bt, int depth, bool forceOpaque, cudaStream_t st, int smCount, uint64_t& launches,
    KernelMarks* marks)
{
    auto mark = [&](int category) {
        if (marks)
            marks->record(category, st);
    };
    int grid = smCount * 8;
    int shadeGrid = smCount * (kShadeMinBlocks > 8 ? kShadeMinBlocks : 8);
    int traceGrid = smCount * kTraceBlocksPerSM;
    mark(KC_CAMERA);
    k_camera<kBatch><<<grid, 256, 0, st>>>(f, wp, wb, bt);
    launches++;
    int cur = 0;
    size_t stackBytes = kTraceStackBytes;
    for (int b = 0; b <= depth; b++)
    {
        if (b == depth)
        {
            mark(KC_SHADE);
            if (!kBatch && s.matGraph)
                k_shade<false, true><<<shadeGrid, kShadeBlock, 0, st>>>(s, f, wp, wb, b, cur, 1, bt);
            else
                k_shade<kBatch><<<shadeGrid, kShadeBlock, 0, st>>>(s, f, wp, wb, b, cur, 1, bt);
            launches++;
            break;
        }
        mark(KC_CLOSEST);
        if (wp.countTraversal)
            k_trace_closest<true, kBatch><<<traceGrid, kTraceBlock, stackBytes, st>>>(s, wb, b, cur, bt);
        else
            k_trace_closest<false, kBatch><<<traceGrid, kTraceBlock, stackBytes, st>>>(s, wb, b, cur, bt);
        if (!kBatch && s.ground.enabled)
        {
            // Ground plane for the bounce's primary rays before they are shaded.
            mark(KC_SHADE);
            k_ground<<<grid, 256, 0, st>>>(s, f, wp, wb, b, cur);
            mark(KC_SHADOW);
            if (wp.countTraversal)
                k_trace_shadow<true, false><<<traceGrid, kTraceBlock, stackBytes, st>>>(s, wb, b,
                    CNT_GROUND_SHADOW, CNT_GROUND_WORK, bt);
            else
                k_trace_shadow<false, false><<<traceGrid, kTraceBlock, stackBytes, st>>>(s, wb, b,
                    CNT_GROUND_SHADOW, CNT_GROUND_WORK, bt);
            mark(KC_SHADE);
            k_ground_shadow<<<grid, 256, 0, st>>>(s, wb, b);
            launches += 3;
        }
        mark(KC_SHADE);
        if (!kBatch && s.matGraph)
            k_shade<false, true><<<shadeGrid, kShadeBlock, 0, st>>>(s, f, wp, wb, b, cur, 0, bt);
        else
            k_shade<kBatch><<<shadeGrid, kShadeBlock, 0, st>>>(s, f, wp, wb, b, cur, 0, bt);
        mark(KC_SHADE);
        k_shade_scatter<kBatch><<<shadeGrid, kShadeBlock, 0, st>>>(s, f, wp, wb, b, cur, bt);
        mark(KC_SHADE);
        k_shade_mis<kBatch><<<shadeGrid, kShadeBlock, 0, st>>>(s, f, wp, wb, b, bt);
        mark(KC_SHADOW);
        if (!forceOpaque)
        {
            if (wp.countTraversal)
                k_trace_shadow_transparent<true, kBatch><<<traceGrid, kTraceBlock, stackBytes, st>>>(s, wb, b, bt);
            else
                k_trace_shadow_transparent<false, kBatch><<<traceGrid, kTraceBlock, stackBytes, st>>>(s, wb, b, bt);
        }
        else if (wp.countTraversal)
            k_trace_shadow<true, kBatch><<<traceGrid, kTraceBlock, stackBytes, st>>>(s, wb, b, CNT_SHADOW,
                CNT_SHADOW_WORK, bt);
        else
            k_trace_shadow<false, kBatch><<<traceGrid, kTraceBlock, stackBytes, st>>>(s, wb, b, CNT_SHADOW,
                CNT_SHADOW_WORK, bt);
        mark(KC_RESOLVE);
        k_resolve<kBatch><<<grid, 256, 0, st>>>(f, wb, b, bt);
        launches += 6;
        if (!kBatch && wp.binRays && b + 1 < depth)
        {
            // The next bounce's rays, binned from queue cur ^ 1 back into queue cur (free since
            // this bounce's shading).
            mark(KC_RESOLVE);
            k_bin_count<<<grid, 256, 0, st>>>(wp, wb, b + 1, cur ^ 1);
            k_bin_scan<<<1, 1024, 0, st>>>(wb);
            k_bin_scatter<<<grid, 256, 0, st>>>(wp, wb, b + 1, cur ^ 1);
            launches += 3;
        }
        else
            cur ^= 1;
    }
    mark(KC_FINALIZE);
#if AGB_SAMPLE_INNER
    if (!kBatch)
        k_finalize_staged<<<grid, 256, 0, st>>>(f, wp, wb);
    else
#endif
        k_finalize<kBatch><<<grid, 256, 0, st>>>(f, wp, wb, bt);
    launches++;
    mark(KC_END);
}

__global__ void k_vertex_records(const float* pos, const float* nrm, const float* uv, uint32_t n, float4* out)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
    {
        const float nx = nrm ? nrm[3 * size_t(i)] : 0.f, ny = nrm ? nrm[3 * size_t(i) + 1] : 0.f,
                    nz = nrm ? nrm[3 * size_t(i) + 2] : 0.f;
        const float u = uv ? uv[2 * size_t(i)] : 0.f, v = uv ? uv[2 * size_t(i) + 1] : 0.f;
        out[2 * size_t(i)]     = make_float4(pos[3 * size_t(i)], pos[3 * size_t(i) + 1], pos[3 * size_t(i) + 2], nx);
        out[2 * size_t(i) + 1] = make_float4(ny, nz, u, v);
    }
}

cudaError_t launchVertexRecords(const float* positions, const float* normals, const float* texcoords,
    uint32_t vertexCount, float4* verts, cudaStream_t stream)
{
    if (vertexCount == 0)
        return cudaSuccess;
    const uint32_t blocks = std::min<uint32_t>((vertexCount + 255) / 256, 65535u);
    k_vertex_records<<<blocks, 256, 0, stream>>>(positions, normals, texcoords, vertexCount, verts);
    return cudaGetLastError();
}

void launchWave(const DevScene& s, const agb_frame_data& f, const WaveParams& wp,
    const WaveBuffers& wb, cudaStream_t st, int smCount, uint64_t& launches, KernelMarks* marks)
{
    BatchTables none{};
    launchWaveT<false>(s, f, wp, wb, none, f.trace_depth, f.is_force_opaque_shadows_enabled != 0, st, smCount,
        launches, marks);
}

void launchBatchWave(const DevScene& shared, const agb_frame_data& anyFrame, const WaveParams& wp,
    const WaveBuffers& wb, const BatchTables& bt, int maxDepth, bool forceOpaque, cudaStream_t st, int smCount,
    uint64_t& launches, KernelMarks* marks)
{
    launchWaveT<true>(shared, anyFrame, wp, wb, bt, maxDepth, forceOpaque, st, smCount, launches, marks);
}

template <class K>
void traceAttributes(K kernel, int stackBytes, int carveout)
{
    cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, stackBytes);
    cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, carveout);
}

void setTraceAttributes()
{
    int stackBytes = int(kTraceStackBytes);
    int carveout   = traceCarveoutPercent();
    traceAttributes(k_trace_closest<true, false>, stackBytes, carveout);
    traceAttributes(k_trace_closest<false, false>, stackBytes, carveout);
    traceAttributes(k_trace_closest<true, true>, stackBytes, carveout);
    traceAttributes(k_trace_closest<false, true>, stackBytes, carveout);
    traceAttributes(k_trace_shadow<true, false>, stackBytes, carveout);
    traceAttributes(k_trace_shadow<false, false>, stackBytes, carveout);
    traceAttributes(k_trace_shadow<true, true>, stackBytes, carveout);
    traceAttributes(k_trace_shadow<false, true>, stackBytes, carveout);
    traceAttributes(k_trace_shadow_transparent<true, false>, stackBytes, carveout);
    traceAttributes(k_trace_shadow_transparent<false, false>, stackBytes, carveout);
    traceAttributes(k_trace_shadow_transparent<true, true>, stackBytes, carveout);
    traceAttributes(k_trace_shadow_transparent<false, true>, stackBytes, carveout);
}

} // namespace agb
