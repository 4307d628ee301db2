// Wavefront path-tracer state: the per-path and per-queue arrays that live in HBM between the
// kernels of one wave.  A wave holds `samples` consecutive sample indices for every pixel; with
// the samples of a pixel side by side (the default), path p covers pixel p / samples and sample
// sampleBase + p % samples, so the 32 lanes of a warp start on one pixel's samples.
#pragma once

#include "agb_trace.cuh"

#ifndef AGB_SAMPLE_INNER
#define AGB_SAMPLE_INNER 1
#endif

namespace agb
{

// Path layout within a wave (or a batched request's range of the wave): AGB_SAMPLE_INNER = 1
// puts a pixel's samples in consecutive paths, 0 the pixels of one sample.
AGB_D uint32_t pathPixel(uint32_t local, uint32_t pixels, uint32_t samples)
{
    return AGB_SAMPLE_INNER ? local / samples : local % pixels;
}
AGB_D uint32_t pathSample(uint32_t local, uint32_t pixels, uint32_t samples)
{
    return AGB_SAMPLE_INNER ? local % samples : local / pixels;
}
AGB_D uint32_t pathOf(uint32_t pixel, uint32_t k, uint32_t pixels, uint32_t samples)
{
    return AGB_SAMPLE_INNER ? pixel * samples + k : k * pixels + pixel;
}

constexpr int kShadePointWords = 10; // float4 per shading point handed between the shading kernels
constexpr int kMisWords        = 3;  // float4 of the environment-MIS sample per shading point
constexpr int kMaxShadowSlots = 6; // up to 4 distant lights + 2 environment-MIS rays per hit
// hitInst value of a camera ray absorbed by the ground plane's matte reflection: k_shade skips it.
constexpr int32_t kGroundAbsorbed = -2;

// Per-bounce device counters (kCounterStride words per bounce).
enum : int
{
    CNT_RAYS          = 0, // rays in the bounce's queue
    CNT_SHADOW        = 1, // shadow rays appended by shading
    CNT_RESOLVE       = 2, // paths with a pending record
    CNT_CLOSEST_WORK  = 3, // persistent traversal work counter (closest-hit rays)
    CNT_SHADOW_WORK   = 4, // persistent traversal work counter (shadow rays)
    CNT_SCATTER       = 5, // shading points handed from k_shade to k_shade_scatter
    CNT_GROUND_SHADOW = 6, // ground-plane matte-shadow rays of the bounce's primary rays
    CNT_GROUND_WORK   = 7, // persistent traversal work counter (ground-plane shadow rays)
    kCounterStride    = 8
};

// Path flag bits (mirrors the reference payload bit fields, RayTrace.slang:52-126).
enum : uint32_t
{
    PF_PRIMARY      = 1u << 0,
    PF_ALPHA        = 1u << 1,  // outputAlpha == 1
    PF_INSIDE       = 1u << 2,
    PF_RAYTYPE_SHIFT = 3,       // 5 bits: ray type of the segment being traced
    PF_MISLOBE_SHIFT = 8,       // 5 bits: misLobeID
};
AGB_HD uint32_t pfRayType(uint32_t f) { return (f >> PF_RAYTYPE_SHIFT) & 31u; }
AGB_HD uint32_t pfMisLobe(uint32_t f) { return (f >> PF_MISLOBE_SHIFT) & 31u; }
AGB_HD uint32_t pfSetRayType(uint32_t f, uint32_t t)
{
    return (f & ~(31u << PF_RAYTYPE_SHIFT)) | (t << PF_RAYTYPE_SHIFT);
}
AGB_HD uint32_t pfSetMisLobe(uint32_t f, uint32_t t)
{
    return (f & ~(31u << PF_MISLOBE_SHIFT)) | (t << PF_MISLOBE_SHIFT);
}

// Pending-resolve record bits: which shadow slots carry a contribution and how the segment's
// radiance is routed (RayGen accumulation, MainEntryPoints.slang:160-243).
enum : uint32_t
{
    RS_SLOT_MASK      = 0x3Fu,   // bit k: slot k holds a contribution
    RS_MIS            = 1u << 6, // MIS emitted shadow rays (indirect = mis result)
    RS_DEPTH0         = 1u << 7, // accumulated as the rayDepth == 0 segment
    RS_DIFFUSE_ROUTE  = 1u << 8, // depth 0: misLobeID == DIFFUSE; depth > 0: rayType == DIFFUSE
};

struct WaveBuffers
{
    // Per path.
    uint2* rng;
    float4* contrib;     // rayContribution (xyz)
    uint32_t* flags;
    float4* outDirect;   // xyz direct radiance
    float4* outDiffuse;  // xyz indirect diffuse
    float4* outGlossy;   // xyz indirect glossy
    float4* lastIndirect; // payload.indirect left by the last traced segment (xyz)
    // Pending shadow-ray contributions of the segment shaded at the current bounce.
    float4* pendEmission;   // xyz emission
    float4* pendSegContrib; // xyz rayContribution the segment is scaled by
    float4* pendSlot;       // kMaxShadowSlots per path: xyz contribution
    uint32_t* pendBits;     // RS_* bits
    uint32_t* occluded;     // bit k: shadow slot k occluded
    // Queues.
    float4* rayOrg[2];      // xyz origin, w tmin
    float4* rayDir[2];      // xyz direction, w tmax
    uint32_t* rayPath[2];
    float4* hitTUV;         // t (or -1), u, v, prim (int bits)
    int32_t* hitInst;
    float4* shOrg;
    float4* shDir;
    uint32_t* shTag;        // path << 3 | slot
    uint32_t* resolveList;  // paths with a pending record this bounce
    float4* shadePoint;     // kShadePointWords float4 per shading point, word-major
    float4* misPoint;       // kMisWords float4 per shading point: the environment-MIS sample
    uint32_t* counters;     // per bounce: kCounterStride words (CNT_*)
    uint32_t* binCount;     // kRayBins counts (zero between uses) and their running offsets
    uint32_t* binOffset;
    // Accumulation targets (per pixel).
    float4* accumMean;
    float4* accumSum;
    float4* accumComp;
    float4* lastSample;
    float2* accumMoments; // sum of luminance, sum of luminance^2
    unsigned long long* stats; // [closest rays, shadow rays, nodes, tris, overflow]
    // Denoising AOVs (per pixel), written for one sample index (WaveParams::aovSample).
    float* aovDepth;     // view-space depth
    float4* aovNormal;   // guide normal xyz, roughness
    float4* aovAlbedo;   // base colour xyz, metalness
    float4* aovMotion;   // previous - current pixel xy, view depth change, 0
};

struct WaveParams
{
    uint32_t width, height, pixels;
    uint32_t sampleBase, samples; // this wave
    uint32_t paths;               // pixels * samples
    uint32_t accumMode;           // AGB_ACCUM_* bits
    int32_t countTraversal;
    uint32_t aovSample;           // sample index whose primary paths write the AOVs; ~0u = none
    uint32_t seedOffset;          // added to the sample index that seeds the random streams
    // Ray binning between bounces (binRays != 0): the next bounce's rays are regrouped by their
    // origin's cell in a 16^3 grid over the scene bounds and their direction octant.
    int32_t binRays;
    float binLo[3];
    float binScale[3];            // cells per unit along each axis
};

constexpr int kRayBinBits = 15;   // 3 bits of octant above a 12-bit Morton cell index
constexpr uint32_t kRayBins = 1u << kRayBinBits;

// Batched wavefronts (agb_batch_render): one wave over the paths of several requests, of
// different scenes and resolutions.  Request r owns paths [pathOffset, pathOffset + pixels x
// samples) laid out like a single request's wave (local path = sample x pixels + pixel), so its
// random streams, and therefore its image, are those of the request rendered alone.  The scenes
// of a batch share one device namespace (meshes, instances, TLAS nodes, materials, images and
// layers concatenated, indices offset); each scene-table entry carries that namespace plus the
// scene's own TLAS root, environment and ground plane.
struct BatchRequest
{
    uint32_t pathOffset, pixelOffset, pixels, width;
    uint32_t height, sampleBase, samples, aovSample;
    uint32_t seedOffset, accumMode;
    int32_t scene;      // index into BatchTables::scenes
    int32_t traceDepth; // the request's frame trace depth
    int32_t tlasRoot;   // the scene's TLAS root in the shared namespace (kDone: no instances)
    int32_t _pad[3];
    float4* accumMean;
    float4* accumSum;
    float4* accumComp;
    float4* lastSample;
    float2* accumMoments;
    float* aovDepth;
    float4* aovNormal;
    float4* aovAlbedo;
    float4* aovMotion;
};

struct BatchTables
{
    const BatchRequest* req;      // null: a single-request wave
    const agb_frame_data* frames; // one per request
    const DevScene* scenes;
    uint16_t* pathReq;            // request index per path
    uint32_t requestCount;
    uint32_t pixelsTotal;         // sum of the requests' pixels (finalize)
};

// Request owning path p (requests sorted by pathOffset; a short binary search over the table).
AGB_D uint32_t batchRequestOfPath(const BatchTables& bt, uint32_t p)
{
    uint32_t lo = 0, hi = bt.requestCount;
    while (hi - lo > 1)
    {
        uint32_t mid = (lo + hi) >> 1;
        if (bt.req[mid].pathOffset <= p)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}
AGB_D uint32_t batchRequestOfPixel(const BatchTables& bt, uint32_t q)
{
    uint32_t lo = 0, hi = bt.requestCount;
    while (hi - lo > 1)
    {
        uint32_t mid = (lo + hi) >> 1;
        if (bt.req[mid].pixelOffset <= q)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

} // namespace agb
